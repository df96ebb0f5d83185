"""CPU-side parity of the product's host Tier-2 (packet headers with tag
trees, Table B-4 pass counts, Lblock comma codes and 0xFF stuffing; SIZ, COD,
QCD, SOT, SOD, EOC; JP2 boxes) against the oracle's restatement of
src/encode/backend/native/t2.rs:337-473, src/j2k/write.rs:9-77 and
src/jp2.rs:13-71, on random per-block retained data, and of its encoding
plan. No GPU: both sides take the same inputs."""
import numpy as np
import pytest

from jp2lam_gb300 import _native


def _block_count(orc, w, h, ncomp, quality):
    """Code-blocks of a page: every band of every resolution split into
    code-blocks (src/encode/backend/native/layout.rs:120-159)."""
    plan = orc.plan(w, h, ncomp, quality)
    cb = plan["cbw"]
    rw, rh, dims = w, h, []
    for _ in range(plan["levels"]):
        lw, hw, lh, hh = (rw + 1) // 2, rw // 2, (rh + 1) // 2, rh // 2
        dims += [(hw, lh), (lw, hh), (hw, hh)]
        rw, rh = lw, lh
    dims.append((rw, rh))
    return ncomp * sum(((bw + cb - 1) // cb) * ((bh + cb - 1) // cb) for bw, bh in dims if bw > 0 and bh > 0)


def _records(n, seed, long_segments=False):
    rng = np.random.default_rng(seed)
    kind = rng.integers(0, 20, n)
    npasses = np.where(kind < 5, 0, np.where(kind < 18, rng.integers(1, 41, n), rng.integers(41, 165, n)))
    zbp = rng.integers(0, 26, n)
    top = 70000 if long_segments else 3000
    seg = np.where(rng.integers(0, 10, n) == 0, 0, rng.integers(1, top, n))
    seg = np.where(npasses > 0, seg, 0)
    body = rng.integers(0, 256, int(seg.sum()), dtype=np.uint8)
    return npasses.astype(np.uint16), zbp.astype(np.uint8), seg.astype(np.uint32), body


@pytest.mark.parametrize("w,h,ncomp,quality,fmt", [
    (1, 1, 1, 85, 0), (7, 33, 3, 50, 1), (64, 64, 1, 100, 0), (100, 70, 3, 99, 1),
    (257, 129, 1, 20, 0), (300, 257, 3, 29, 1), (512, 512, 1, 85, 1), (1275, 1650, 3, 75, 1),
])
def test_host_tier2_matches_oracle(orc, w, h, ncomp, quality, fmt):
    n = _block_count(orc, w, h, ncomp, quality)
    for seed in range(3):
        rec = _records(n, 100 * w + seed, long_segments=seed == 2)
        got = _native.debug_assemble(w, h, ncomp, quality, fmt, *rec)
        want = orc.assemble(w, h, ncomp, quality, fmt, *rec)
        assert got == want


def test_host_tier2_rejects_a_wrong_block_count(orc):
    n = _block_count(orc, 100, 70, 1, 85)
    rec = _records(n + 1, 5)
    with pytest.raises(_native.InvalidInput):
        _native.debug_assemble(100, 70, 1, 85, 0, *rec)


@pytest.mark.parametrize("w,h,ncomp", [(1, 1, 1), (7, 33, 3), (64, 64, 1), (300, 257, 3), (2550, 3300, 1),
                                        (2550, 3300, 3), (5100, 6600, 3), (256, 256, 1), (33, 1000, 1)])
@pytest.mark.parametrize("quality", [0, 1, 20, 29, 30, 50, 60, 75, 85, 90, 99, 100, 101, 255])
def test_host_plan_matches_oracle(orc, w, h, ncomp, quality):
    # levels, code-block size, quantiser entries (norms.rs:68-90,
    # derive.rs:60-165), code-block count and the PCRD lambdas
    # (pcrd.rs:1425-1456) that the device kernels are driven by
    got = _native.debug_plan(w, h, ncomp, quality)
    want = orc.plan(w, h, ncomp, quality)
    assert got["levels"] == want["levels"]
    assert got["cbw"] == want["cbw"]
    assert [tuple(int(v) for v in q) for q in got["quants"]] == [tuple(int(v) for v in q) for q in want["quants"]]
    assert got["nblocks"] == _block_count(orc, w, h, ncomp, quality)
    f = orc.lib.orc_quality_to_lambda
    assert got["lambdas"] == (f(quality, w * h), f(1, w * h))
