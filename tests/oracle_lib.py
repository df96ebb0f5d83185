"""ctypes binding of the oracle (oracle/_build/liborc.so).

The oracle is the CPU restatement of the reference encoder; it is the checker
the CUDA path is compared against and is used only by tests, smoke() and the
CPU-baseline leg of bench.py.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_build", "liborc.so")

_u8p = ctypes.POINTER(ctypes.c_uint8)


class Oracle:
    def __init__(self, lib):
        self.lib = lib
        lib.orc_last_error.restype = ctypes.c_char_p
        lib.orc_quality_to_lambda.restype = ctypes.c_double
        lib.orc_norm97.restype = ctypes.c_double
        lib.orc_time_encode.restype = ctypes.c_double
        lib.orc_mq_encode.restype = _u8p

    def _err(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: code {rc}: {self.lib.orc_last_error().decode()}")

    def encode(self, px, w, h, ncomp, quality, fmt=0, threads=1, contrast_mask=False):
        px = np.ascontiguousarray(px, dtype=np.uint8)
        out = _u8p()
        n = ctypes.c_size_t()
        rc = self.lib.orc_encode(px.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint32(w),
                                 ctypes.c_uint32(h), ncomp, quality, fmt, threads,
                                 int(contrast_mask), ctypes.byref(out), ctypes.byref(n))
        self._err(rc, "orc_encode")
        data = ctypes.string_at(out, n.value)
        self.lib.orc_free(out)
        return data

    def assemble(self, w, h, ncomp, quality, fmt, npasses, zbp, seg_len, body):
        """Tier-2, markers and JP2 boxes from per-block retained data in
        codestream order (the oracle's own layout geometry)."""
        npasses = np.ascontiguousarray(npasses, dtype=np.uint16)
        zbp = np.ascontiguousarray(zbp, dtype=np.uint8)
        seg_len = np.ascontiguousarray(seg_len, dtype=np.uint32)
        body = np.ascontiguousarray(body, dtype=np.uint8)
        out = _u8p()
        n = ctypes.c_size_t()
        ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        rc = self.lib.orc_assemble(ctypes.c_uint32(w), ctypes.c_uint32(h), ncomp, quality, fmt, ptr(npasses),
                                   ptr(zbp), ptr(seg_len), ptr(body) if body.size else None,
                                   ctypes.c_uint32(len(npasses)), ctypes.byref(out), ctypes.byref(n))
        self._err(rc, "orc_assemble")
        data = ctypes.string_at(out, n.value)
        self.lib.orc_free(out)
        return data

    def coefficients(self, px, w, h, ncomp, quality, comp):
        px = np.ascontiguousarray(px, dtype=np.uint8)
        out = np.zeros(w * h, np.int32)
        rc = self.lib.orc_coefficients(px.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint32(w),
                                       ctypes.c_uint32(h), ncomp, quality, comp,
                                       out.ctypes.data_as(ctypes.c_void_p))
        self._err(rc, "orc_coefficients")
        return out.reshape(h, w)

    def coefficients_f64(self, px, w, h, ncomp, quality, comp):
        """(FP64 9/7 coefficients, quantiser steps, the f32 restatement's
        unquantised coefficients) of one component, each h x w."""
        px = np.ascontiguousarray(px, dtype=np.uint8)
        c64 = np.zeros(w * h, np.float64)
        st = np.zeros(w * h, np.float32)
        f32 = np.zeros(w * h, np.float32)
        ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        rc = self.lib.orc_coefficients_f64(ptr(px), ctypes.c_uint32(w), ctypes.c_uint32(h), ncomp, quality, comp,
                                           ptr(c64), ptr(st), ptr(f32))
        self._err(rc, "orc_coefficients_f64")
        return c64.reshape(h, w), st.reshape(h, w), f32.reshape(h, w)

    def plan(self, w, h, ncomp, quality):
        lv, cbw, nq = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        q = np.zeros(4 * 32, np.int32)
        rc = self.lib.orc_plan(ctypes.c_uint32(w), ctypes.c_uint32(h), ncomp, quality,
                               ctypes.byref(lv), ctypes.byref(cbw), ctypes.byref(nq),
                               q.ctypes.data_as(ctypes.c_void_p))
        self._err(rc, "orc_plan")
        return {"levels": lv.value, "cbw": cbw.value,
                "quants": [tuple(q[4 * i:4 * i + 4]) for i in range(nq.value)]}

    def dwt(self, data, w, h, levels, kind, inverse=False):
        if kind == 53:
            a = np.ascontiguousarray(data, dtype=np.int32).copy()
            f = self.lib.orc_inv53 if inverse else self.lib.orc_fwd53
        else:
            a = np.ascontiguousarray(data, dtype=np.float32).copy()
            f = self.lib.orc_inv97 if inverse else self.lib.orc_fwd97
        f(a.ctypes.data_as(ctypes.c_void_p), w, h, levels)
        return a

    def tables(self):
        zc = np.zeros(2048, np.uint8)
        sc = np.zeros(256, np.uint8)
        spb = np.zeros(256, np.uint8)
        mq = np.zeros(94 * 4, np.uint16)
        self.lib.orc_tables(*(a.ctypes.data_as(ctypes.c_void_p) for a in (zc, sc, spb, mq)))
        return zc, sc, spb, mq

    def mq_encode(self, syms, variant=0):
        syms = np.ascontiguousarray(syms, dtype=np.uint8)
        n = ctypes.c_size_t()
        p = self.lib.orc_mq_encode(syms.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(syms.size),
                                   variant, ctypes.byref(n))
        data = ctypes.string_at(p, n.value)
        self.lib.orc_free(p)
        return data

    def mq_decode(self, data, ctxs):
        ctxs = np.ascontiguousarray(ctxs, dtype=np.uint8)
        bits = np.zeros(ctxs.size, np.uint8)
        self.lib.orc_mq_decode(data, ctypes.c_size_t(len(data)), ctxs.ctypes.data_as(ctypes.c_void_p),
                               ctypes.c_size_t(ctxs.size), bits.ctypes.data_as(ctypes.c_void_p))
        return bits

    def t1_block(self, coefs, w, h, band, mb):
        coefs = np.ascontiguousarray(coefs, dtype=np.int32)
        mbp, zbp, cls, npasses = (ctypes.c_int() for _ in range(4))
        cap = 128
        passes = np.zeros(6 * cap, np.int32)
        out = _u8p()
        n = ctypes.c_size_t()
        rc = self.lib.orc_t1_block(coefs.ctypes.data_as(ctypes.c_void_p), w, h, band, mb,
                                   ctypes.byref(mbp), ctypes.byref(zbp), ctypes.byref(cls),
                                   ctypes.byref(npasses), passes.ctypes.data_as(ctypes.c_void_p),
                                   cap, ctypes.byref(out), ctypes.byref(n))
        self._err(rc, "orc_t1_block")
        payload = ctypes.string_at(out, n.value)
        self.lib.orc_free(out)
        return {"mbp": mbp.value, "zbp": zbp.value, "cls": cls.value,
                "passes": passes[:6 * npasses.value].reshape(-1, 6), "payload": payload}

    def t1_decode(self, data, w, h, band, mb, zbp, npasses):
        out = np.zeros(w * h, np.int32)
        rc = self.lib.orc_t1_decode(data, ctypes.c_size_t(len(data)), w, h, band, mb, zbp, npasses,
                                    out.ctypes.data_as(ctypes.c_void_p))
        if rc != 0:
            raise RuntimeError(f"orc_t1_decode: code {rc}")
        return out

    def block_summary(self, px, w, h, ncomp, quality, pcrd=True):
        px = np.ascontiguousarray(px, dtype=np.uint8)
        cap = 1 << 20
        rows = np.zeros(9 * cap, np.int32)
        n = ctypes.c_int()
        rc = self.lib.orc_block_summary(px.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint32(w),
                                        ctypes.c_uint32(h), ncomp, quality, int(pcrd),
                                        rows.ctypes.data_as(ctypes.c_void_p), cap, ctypes.byref(n))
        self._err(rc, "orc_block_summary")
        return rows[:9 * n.value].reshape(-1, 9)

    def decode(self, data, rct_chroma_extra_bitplane=False, accept_empty_segments=False):
        """The reference's decoder (src/decode/*.rs); with
        rct_chroma_extra_bitplane, RCT chroma code-blocks are read with the
        extra bit-plane their encoder gave them (backend.rs:179-189), which
        the reference's decoder does not do; with accept_empty_segments, a
        code-block with passes but no bytes is decoded from an all-0xFF
        stream instead of rejected (decode/t1.rs:109-111)."""
        w, h, c = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_int()
        flag = int(bool(rct_chroma_extra_bitplane)) | (2 if accept_empty_segments else 0)
        rc = self.lib.orc_decode_ex(data, ctypes.c_size_t(len(data)), flag, ctypes.byref(w), ctypes.byref(h),
                                    ctypes.byref(c), None, ctypes.c_size_t(0))
        self._err(rc, "orc_decode")
        px = np.zeros(w.value * h.value * c.value, np.uint8)
        rc = self.lib.orc_decode_ex(data, ctypes.c_size_t(len(data)), flag, ctypes.byref(w), ctypes.byref(h),
                                    ctypes.byref(c), px.ctypes.data_as(ctypes.c_void_p),
                                    ctypes.c_size_t(px.size))
        self._err(rc, "orc_decode")
        return w.value, h.value, c.value, px

    def frame(self, w, h, ncomp, quality, main, tile_hdr, payload, tile=0, part=0, parts=0):
        """Codestream framing alone (src/j2k/write.rs:9-113): SOC, the
        main-header segments `main`, one tile-part with header segments
        `tile_hdr` and `payload`, EOC; under the plan of a w x h page."""
        out = _u8p()
        n = ctypes.c_size_t()
        rc = self.lib.orc_frame(ctypes.c_uint32(w), ctypes.c_uint32(h), ncomp, quality, bytes(main),
                                ctypes.c_size_t(len(main)), bytes(tile_hdr), ctypes.c_size_t(len(tile_hdr)),
                                tile, part, parts, bytes(payload), ctypes.c_size_t(len(payload)),
                                ctypes.byref(out), ctypes.byref(n))
        self._err(rc, "orc_frame")
        data = ctypes.string_at(out, n.value)
        self.lib.orc_free(out)
        return data

    def reframe(self, cs, w, h, ncomp, quality):
        """Parses a single-tile codestream and frames it again."""
        out = _u8p()
        n = ctypes.c_size_t()
        rc = self.lib.orc_reframe(bytes(cs), ctypes.c_size_t(len(cs)), ctypes.c_uint32(w), ctypes.c_uint32(h),
                                  ncomp, quality, ctypes.byref(out), ctypes.byref(n))
        self._err(rc, "orc_reframe")
        data = ctypes.string_at(out, n.value)
        self.lib.orc_free(out)
        return data

    def quality_metrics(self, px, w, h, ncomp, quality):
        px = np.ascontiguousarray(px, dtype=np.uint8)
        psnr, ssim = ctypes.c_double(), ctypes.c_double()
        rc = self.lib.orc_quality_metrics(px.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint32(w),
                                          ctypes.c_uint32(h), ncomp, quality, ctypes.byref(psnr),
                                          ctypes.byref(ssim))
        self._err(rc, "orc_quality_metrics")
        return psnr.value, ssim.value

    def time_encode(self, px, w, h, ncomp, quality, fmt, threads, contrast_mask, iters):
        px = np.ascontiguousarray(px, dtype=np.uint8)
        return self.lib.orc_time_encode(px.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint32(w),
                                        ctypes.c_uint32(h), ncomp, quality, fmt, threads,
                                        int(contrast_mask), iters)


def build():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)


_cached = None


def load():
    global _cached
    if _cached is None:
        if not os.path.exists(LIB):
            build()
        _cached = Oracle(ctypes.CDLL(LIB))
    return _cached
