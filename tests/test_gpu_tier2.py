"""Device Tier-2 against the host Tier-2 and the oracle, byte for byte.

The encoder writes packet headers (tag trees, Table B-4 pass counts, Lblock
comma codes, 0xFF bit stuffing), markers and JP2 boxes on the device
(t2dev.cu); jp2g_debug_assemble_device runs those kernels on given per-block
records. Random records cover empty blocks, 1-164 passes, zero bit-plane
counts up to 25 and segments up to 70,000 bytes; a second set makes headers
with long runs of one bits so that the stuffing after 0xFF bytes is
exercised, including a header that ends in 0xFF. Whole-page parity of the
encoder (which now always assembles on the device) is covered by the other
GPU parity tests."""
import numpy as np
import pytest

import jp2lam_gb300 as jl
from jp2lam_gb300 import _native
from tests.test_host_tier2 import _block_count, _records

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 1, 85, 0), (7, 33, 3, 50, 1), (64, 64, 1, 100, 0), (100, 70, 3, 99, 1), (257, 129, 1, 20, 0),
          (300, 257, 3, 29, 1), (512, 512, 1, 85, 1), (1275, 1650, 3, 75, 1), (2550, 3300, 1, 85, 1),
          (3400, 4400, 3, 50, 1), (33, 1000, 1, 60, 0), (1000, 33, 3, 100, 1)]


@pytest.fixture(scope="module")
def eng():
    e = jl.Engine(0)
    yield e
    e.close()


@pytest.mark.parametrize("w,h,ncomp,quality,fmt", SHAPES)
def test_device_tier2_matches_host_and_oracle(eng, orc, w, h, ncomp, quality, fmt):
    n = _block_count(orc, w, h, ncomp, quality)
    for seed in range(3):
        rec = _records(n, 7 * w + h + seed, long_segments=seed == 2)
        got = eng.debug_assemble_device(w, h, ncomp, quality, fmt, *rec)
        assert got == _native.debug_assemble(w, h, ncomp, quality, fmt, *rec)
        assert got == orc.assemble(w, h, ncomp, quality, fmt, *rec)


@pytest.mark.parametrize("seed", range(6))
def test_device_tier2_bit_stuffing(eng, orc, seed):
    # every block included with many passes, long segments and zero
    # bit-planes that make runs of ones: many 0xFF header bytes
    w, h, ncomp, quality, fmt = 700, 500, 1, 85, 1
    n = _block_count(orc, w, h, ncomp, quality)
    rng = np.random.default_rng(seed)
    npasses = rng.choice([37, 100, 164, 36, 6], n).astype(np.uint16)
    zbp = rng.choice([0, 1, 25], n).astype(np.uint8)
    seg = rng.choice([65535, 131071, 2 ** 20 - 1, 127, 1], n).astype(np.uint32)
    if seed == 5:
        seg[:] = 255
    body = rng.integers(0, 256, int(seg.sum()), dtype=np.uint8)
    got = eng.debug_assemble_device(w, h, ncomp, quality, fmt, npasses, zbp, seg, body)
    assert got == _native.debug_assemble(w, h, ncomp, quality, fmt, npasses, zbp, seg, body)


def test_device_tier2_rejects_a_wrong_block_count(eng, orc):
    n = _block_count(orc, 100, 70, 1, 85)
    with pytest.raises(jl.InvalidInput):
        eng.debug_assemble_device(100, 70, 1, 85, 0, *_records(n + 1, 5))
