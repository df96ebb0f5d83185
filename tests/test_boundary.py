"""CPU-side checks of the drop-in boundary: the C-ABI library loads and
exports every symbol include/jp2g.h declares, the tables it uploads to the
device equal the reference's, and the host API rejects bad input before any
device work (src/plan/validate.rs:4-62, src/model.rs:87-140)."""
import json
import os
import re

import numpy as np
import pytest

import jp2lam_gb300 as jl
from jp2lam_gb300 import _native
from tests.golden import reference_tables as rt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "jp2g.h")).read()
    return sorted(set(re.findall(r"\b(jp2g_[a-z_0-9]+)\s*\(", hdr)))


def test_library_exports_every_declared_symbol():
    lib = _native.load_library()
    declared = _declared_symbols()
    assert set(declared) == set(_native.EXPORTS)
    for name in declared:
        assert hasattr(lib, name), name


def test_engine_tables_match_reference():
    ref = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_tables.json")))
    zc, sc, spb, mq = _native.tables()
    assert rt.digest(zc) == ref["zc_sha256"]
    assert rt.digest(sc) == ref["sc_sha256"]
    assert rt.digest(spb) == ref["spb_sha256"]
    # expand packed (qe | nmps << 16 | nlps << 24) into (qe, mps, nmps, nlps)
    rows = []
    for i, e in enumerate(mq.tolist()):
        rows += [e & 0xFFFF, i & 1, (e >> 16) & 0xFF, e >> 24]
    assert rt.digest(rows) == ref["mq_states_sha256"]


def test_gray_buffer_length_is_validated():
    with pytest.raises(jl.InvalidInput):
        jl.Image.from_gray_bytes(4, 4, b"\x00" * 15)


def test_rgb_buffer_length_is_validated():
    with pytest.raises(jl.InvalidInput):
        jl.Image.from_rgb_bytes(2, 2, b"\x00" * 11)


def test_zero_dimensions_are_rejected_before_device_work():
    im = jl.Image(0, 4, jl.ColorSpace.GRAY, b"", [jl.Component(0, 4)])
    with pytest.raises(jl.InvalidInput):
        jl.encode(im, jl.EncodeOptions(85, jl.OutputFormat.J2K))


def test_unsupported_precision_is_rejected():
    im = jl.Image.from_gray_bytes(2, 2, b"\x00" * 4)
    im.components[0].precision = 12
    with pytest.raises(jl.InvalidInput):
        jl.encode(im)


def test_batch_encoder_rejects_mismatched_profiles():
    """src/batch.rs:212-221 (profile check happens before encoding)."""
    enc = jl.BatchEncoder(jl.EncodeOptions())
    a = jl.Image.from_gray_bytes(2, 2, b"\x80" * 4)
    b = jl.Image.from_gray_bytes(3, 2, b"\x80" * 6)
    enc._validate_or_set_profile(a)
    enc._validate_or_set_profile(a)
    with pytest.raises(jl.InvalidInput):
        enc._validate_or_set_profile(b)


def test_presets_and_defaults():
    """src/model.rs:41-62, 169-177"""
    assert jl.Preset.DOCUMENT_LOW.quality() == 30
    assert jl.Preset.DOCUMENT_HIGH.quality() == 85
    assert jl.Preset.WEB_LOW.quality() == 42
    assert jl.Preset.WEB_HIGH.quality() == 62
    o = jl.EncodeOptions()
    assert o.quality == 85 and o.format == jl.OutputFormat.JP2


def test_no_cpu_fallback_without_gpu():
    """Creating an engine on a machine without a usable GPU fails loudly."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(jl.Jp2LamError):
        jl.Engine(0)


def test_synthetic_page_is_deterministic():
    a = _native.synth_page(512, 512, 1, 0, glyphs=400)
    b = _native.synth_page(512, 512, 1, 0, glyphs=400)
    assert np.array_equal(a, b)
    assert a.min() >= 10 and a.max() <= 248
    bg = a[(a >= 242)]
    assert bg.size > 0.6 * a.size
    c = _native.synth_page(256, 192, 3, 5, photo_w=120, photo_h=90)
    assert c.size == 256 * 192 * 3


def test_bit_sliced_context_logic_equals_the_context_tables():
    # the modelling kernel forms zero-coding labels, sign contexts and sign
    # predictions with bit-sliced logic; on every neighbourhood it must give
    # the tables' entries (which equal the reference's literal tables)
    zc, sc, spb, _ = _native.tables()
    lz, ls, lp = _native.context_labels()
    for o in range(4):
        for f in range(512):
            assert lz[o * 512 + f] == zc[o * 512 + f], (o, f)
    assert np.array_equal(ls, sc)
    assert np.array_equal(lp, spb)
