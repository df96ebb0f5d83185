"""GPU test of jp2g_dwt_noalloc, the allocation-free entry point.

That entry point serves callers that cannot allocate device memory (code
recorded into CUDA graphs, hosts that only lend pre-allocated buffers,
loops that must not call the allocator). It keeps its scratch in a static
device array instead of calling cudaMalloc, so this test checks that its
coefficients match what the regular encoder computes (bit-exact, the
tolerance of every integer parity test here), twice in a row on the same
shared scratch, and that oversized images are refused before any device
work. The file is named to run last.
"""
import ctypes

import numpy as np
import pytest

import jp2lam_gb300 as jl
from jp2lam_gb300 import _native
from jp2lam_gb300._native import synth_page

pytestmark = pytest.mark.gpu

# the last two: a reversible quality above 100 (every quality >= 100 takes
# the 5/3 path), and an image exactly at the scratch limit
# (ceil(w/2) * ceil(h/2) * ncomp = 1,048,576)
CASES = [(700, 500, 3, 85), (640, 480, 1, 100), (257, 129, 1, 20), (96, 64, 3, 100), (7, 5, 1, 50),
         (1, 9, 3, 85), (200, 150, 3, 180), (2048, 2048, 1, 85)]


def _noalloc(lib, d_px, w, h, c, q, d_out, stream):
    return lib.jp2g_dwt_noalloc(ctypes.c_void_p(d_px.data_ptr()), w, h, c, q,
                                ctypes.c_void_p(d_out.data_ptr()), ctypes.c_void_p(stream))


@pytest.mark.parametrize("w,h,c,q", CASES)
def test_noalloc_matches_encoder_coefficients_twice(w, h, c, q):
    import torch
    lib = _native.load_library()
    eng = jl.Engine(0)
    try:
        px = synth_page(w, h, c, w * 7 + h, photo_w=w // 3, photo_h=h // 3)
        want = np.stack([eng.debug_coefficients(px, w, h, c, q, comp) for comp in range(c)])
        d_px = torch.from_numpy(px).cuda()
        d_out = torch.empty(w * h * c, dtype=torch.int32, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        for _ in range(2):
            d_out.fill_(-7)
            rc = _noalloc(lib, d_px, w, h, c, q, d_out, stream)
            assert rc == 0, lib.jp2g_last_error(None).decode()
            torch.cuda.synchronize()
            got = d_out.cpu().numpy().reshape(c, h, w)
            assert np.array_equal(got, want)
    finally:
        eng.close()


def test_noalloc_rejects_images_beyond_its_scratch():
    import torch
    lib = _native.load_library()
    d = torch.empty(16, dtype=torch.int32, device="cuda")
    for w, h, c in ((4096, 4096, 1), (2050, 2048, 1), (1184, 1184, 3)):  # and just past the limit
        rc = lib.jp2g_dwt_noalloc(ctypes.c_void_p(d.data_ptr()), w, h, c, 85,
                                  ctypes.c_void_p(d.data_ptr()), None)
        assert rc == jl.InvalidInput.code
        assert b"allocation-free" in lib.jp2g_last_error(None)
