"""GPU parity at the page shapes the benchmark times, against the oracle.

One full page of each shape the bench measures, encoded through the C ABI
and compared byte for byte with the oracle's codestream on the same pixels:
the 2550x3300 sRGB q75 page of the batched workload, 3400x4400 and 5100x6600
gray and sRGB pages at q50 and q100 and the 1275x1650 pages of the uneven
mix, and the 256x256 gray q60 thumbnail of the served mix (the 2550x3300
gray q85 headline page is in test_gpu_parity.py). A mixed batch of these
pages through jp2g_encode_batch must give each page the oracle's bytes too.
Lossy outputs decode through the oracle's restatement of the reference's
decoder with a PSNR floor; sRGB lossless outputs read back exactly once RCT
chroma gets the extra bit-plane its encoder used (the reference's own
decoder rejects them; the oracle's CPU tests pin that)."""
import numpy as np
import pytest

import jp2lam_gb300 as jl
from jp2lam_gb300._native import synth_page

pytestmark = pytest.mark.gpu

# (name, w, h, ncomp, quality, seed, photo area fraction or fixed photo size)
PAGES = [
    ("srgb_2550x3300_q75", 2550, 3300, 3, 75, 1000, (800, 600)),
    ("gray_3400x4400_q50", 3400, 4400, 1, 50, 2001, 0.30),
    ("gray_3400x4400_q100", 3400, 4400, 1, 100, 2002, 0.10),
    ("srgb_3400x4400_q50", 3400, 4400, 3, 50, 2003, 0.25),
    ("srgb_3400x4400_q100", 3400, 4400, 3, 100, 2004, 0.05),
    ("gray_5100x6600_q50", 5100, 6600, 1, 50, 2005, 0.40),
    ("gray_5100x6600_q100", 5100, 6600, 1, 100, 2006, 0.20),
    ("srgb_5100x6600_q50", 5100, 6600, 3, 50, 2007, 0.15),
    ("srgb_5100x6600_q100", 5100, 6600, 3, 100, 2008, 0.35),
    ("gray_1275x1650_q85", 1275, 1650, 1, 85, 2009, 0.20),
    ("srgb_1275x1650_q75", 1275, 1650, 3, 75, 2010, 0.30),
    ("gray_256x256_q60", 256, 256, 1, 60, 3000, 0.0),
]
IDS = [p[0] for p in PAGES]


def _pixels(spec):
    _, w, h, c, _, seed, photo = spec
    if isinstance(photo, tuple):
        return synth_page(w, h, c, seed, photo_w=photo[0], photo_h=photo[1])
    return synth_page(w, h, c, seed, photo_frac=photo)


class _Cache:
    """Pixels and oracle codestreams, made once per module."""

    def __init__(self, orc):
        self.orc = orc
        self.px = {}
        self.want = {}

    def get(self, spec):
        name, w, h, c, q, _, _ = spec
        if name not in self.px:
            self.px[name] = _pixels(spec)
            self.want[name] = self.orc.encode(self.px[name], w, h, c, q, fmt=1, threads=16)
        return self.px[name], self.want[name]


@pytest.fixture(scope="module")
def cache(orc):
    return _Cache(orc)


@pytest.fixture(scope="module")
def eng():
    e = jl.Engine(0)
    yield e
    e.close()


@pytest.mark.parametrize("spec", PAGES, ids=IDS)
def test_config_page_byte_identical(eng, cache, spec):
    name, w, h, c, q, _, _ = spec
    px, want = cache.get(spec)
    assert eng.encode(px, w, h, c, q, 1) == want


def test_config_pages_in_one_mixed_batch_match_the_oracle(eng, cache):
    # host buffers, every shape and colour at once, split into waves by size
    pages = []
    for spec in PAGES:
        name, w, h, c, q, _, _ = spec
        px, _ = cache.get(spec)
        pages.append({"px": px, "w": w, "h": h, "ncomp": c, "quality": q, "fmt": 1})
    outs = eng.encode_batch(pages)
    for spec, out in zip(PAGES, outs):
        assert out == cache.get(spec)[1], spec[0]


@pytest.mark.parametrize("spec", [PAGES[0], PAGES[-1], PAGES[4], PAGES[10]],
                         ids=[PAGES[0][0], PAGES[-1][0], PAGES[4][0], PAGES[10][0]])
def test_config_page_decodes(cache, spec):
    name, w, h, c, q, _, _ = spec
    px, data = cache.get(spec)
    orc = cache.orc
    dw, dh, dc, dec = orc.decode(data, rct_chroma_extra_bitplane=(c == 3 and q >= 100))
    assert (dw, dh, dc) == (w, h, c)
    if q >= 100:
        assert np.array_equal(dec, px)
    else:
        mse = np.mean((dec.astype(np.float64) - px) ** 2)
        assert 10 * np.log10(255.0 ** 2 / mse) > 28.0
