"""ctypes binding of libjp2g.so (the C ABI declared in include/jp2g.h).

The library is built in-tree by jp2lam_gb300/build.py. Loading never falls
back to anything else: a missing library or a missing GPU raises.
"""
from __future__ import annotations

import ctypes
import weakref
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libjp2g.so")
SYNTH_PATH = os.path.join(HERE, "_lib", "libjp2g_synth.so")

_u8p = ctypes.POINTER(ctypes.c_uint8)


class Jp2LamError(Exception):
    """Base of the reference's error variants (src/error.rs:7-13)."""
    code = 2


class InvalidInput(Jp2LamError):
    code = 1


class EncodeFailed(Jp2LamError):
    code = 2


class DecodeFailed(Jp2LamError):
    code = 3


class UnsupportedFeature(Jp2LamError):
    code = 4


class IoError(Jp2LamError):
    code = 5


_BY_CODE = {1: InvalidInput, 2: EncodeFailed, 3: DecodeFailed, 4: UnsupportedFeature, 5: IoError}

# Every symbol the header declares (checked by the CPU test-suite).
EXPORTS = [
    "jp2g_create", "jp2g_destroy", "jp2g_encode", "jp2g_encode_device", "jp2g_free",
    "jp2g_last_error", "jp2g_stream", "jp2g_set_timing", "jp2g_stage_times", "jp2g_counters",
    "jp2g_debug_coefficients", "jp2g_debug_blocks", "jp2g_dwt_noalloc", "jp2g_tables",
    "jp2g_encode_batch", "jp2g_submit", "jp2g_poll", "jp2g_set_option", "jp2g_get_option",
    "jp2g_autotune", "jp2g_debug_assemble", "jp2g_debug_plan", "jp2g_cancel", "jp2g_debug_context_labels",
    "jp2g_debug_coefficients_f32", "jp2g_encode_with_psnr", "jp2g_debug_assemble_device", "jp2g_decode",
    "jp2g_decode_batch",
]

PENDING = 6
OPT_WAVE_BLOCKS = 0
OPT_MQ_BLOCKS_PER_WARP = 1
OPT_HOST_THREADS = 2
OPT_MQ_WARPS_PER_SM = 3
OPT_MQ_PIPES_PER_SM = 4
OPT_MQ_HEAVY = 5
OPT_MQ_CHAINS_PER_PAIR = 6
NUM_OPTS = 7


class Request(ctypes.Structure):
    """jp2g_request: one page of a batch or a served request."""
    _fields_ = [("px", ctypes.c_void_p), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("ncomp", ctypes.c_uint32), ("interleaved", ctypes.c_int32), ("on_device", ctypes.c_int32),
                ("quality", ctypes.c_int32), ("format", ctypes.c_int32)]

_lib = None
_lock = threading.Lock()
_engine_lock = threading.Lock()


def load_library(path: str = LIB_PATH):
    """Loads libjp2g.so and declares its signatures. Raises if it is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise EncodeFailed(f"CUDA engine library not built: {path} (run jp2lam_gb300/build.py)")
        lib = ctypes.CDLL(path)
        lib.jp2g_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_uint64]
        lib.jp2g_destroy.argtypes = [ctypes.c_void_p]
        lib.jp2g_encode.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_uint32, ctypes.c_int, ctypes.c_uint8, ctypes.c_int,
                                    ctypes.POINTER(_u8p), ctypes.POINTER(ctypes.c_size_t)]
        lib.jp2g_encode_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                           ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint8, ctypes.c_int,
                                           ctypes.POINTER(_u8p), ctypes.POINTER(ctypes.c_size_t)]
        lib.jp2g_free.argtypes = [_u8p]
        lib.jp2g_last_error.argtypes = [ctypes.c_void_p]
        lib.jp2g_last_error.restype = ctypes.c_char_p
        lib.jp2g_stream.argtypes = [ctypes.c_void_p]
        lib.jp2g_stream.restype = ctypes.c_void_p
        lib.jp2g_set_timing.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.jp2g_stage_times.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        lib.jp2g_counters.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        lib.jp2g_debug_coefficients.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                                ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint8,
                                                ctypes.c_uint32, ctypes.c_void_p]
        lib.jp2g_debug_coefficients_f32.argtypes = lib.jp2g_debug_coefficients.argtypes
        lib.jp2g_encode_with_psnr.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32,
                                              ctypes.c_uint32, ctypes.c_int, ctypes.c_uint8, ctypes.c_int,
                                              ctypes.POINTER(_u8p), ctypes.POINTER(ctypes.c_size_t),
                                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        lib.jp2g_decode.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                    ctypes.POINTER(_u8p), ctypes.POINTER(ctypes.c_size_t),
                                    ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                                    ctypes.POINTER(ctypes.c_uint32)]
        lib.jp2g_decode_batch.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                          ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.jp2g_debug_blocks.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                          ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint8,
                                          ctypes.c_void_p, ctypes.c_uint32,
                                          ctypes.POINTER(ctypes.c_uint32)]
        lib.jp2g_tables.argtypes = [ctypes.c_void_p] * 4
        lib.jp2g_dwt_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                         ctypes.c_uint8, ctypes.c_void_p, ctypes.c_void_p]
        lib.jp2g_encode_batch.argtypes = [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.c_uint32,
                                          ctypes.POINTER(_u8p), ctypes.POINTER(ctypes.c_size_t),
                                          ctypes.POINTER(ctypes.c_int)]
        lib.jp2g_submit.argtypes = [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]
        lib.jp2g_poll.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(_u8p),
                                  ctypes.POINTER(ctypes.c_size_t), ctypes.c_int]
        lib.jp2g_cancel.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        lib.jp2g_set_option.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int64]
        lib.jp2g_get_option.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]
        lib.jp2g_autotune.argtypes = [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.c_uint32, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)]
        lib.jp2g_debug_plan.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint8,
                                        ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(ctypes.c_int), ctypes.c_void_p,
                                        ctypes.POINTER(ctypes.c_uint32), ctypes.c_void_p]
        lib.jp2g_debug_assemble.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint8,
                                            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(_u8p),
                                            ctypes.POINTER(ctypes.c_size_t)]
        lib.jp2g_debug_assemble_device.argtypes = [ctypes.c_void_p] + lib.jp2g_debug_assemble.argtypes
        _lib = lib
        return lib


def _raise(code: int, msg: str):
    raise _BY_CODE.get(code, Jp2LamError)(msg)


class Engine:
    """One jp2g context (CUDA stream + device pools) on one GPU."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.jp2g_create(ctypes.byref(h), device, hbm_budget_bytes)
        if rc != 0:
            _raise(rc, self.lib.jp2g_last_error(None).decode())
        self.handle = h
        self._lock = threading.Lock()
        self._inflight = {}  # ticket -> pixel buffer kept alive until polled
        self._inflight_lock = threading.Lock()

    def close(self):
        if getattr(self, "handle", None):
            self.lib.jp2g_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != 0:
            _raise(rc, self.lib.jp2g_last_error(self.handle).decode())

    def encode(self, px, w: int, h: int, ncomp: int, quality: int, fmt: int,
               interleaved: bool = True) -> bytes:
        buf = np.frombuffer(px, dtype=np.uint8) if isinstance(px, (bytes, bytearray)) else \
            np.ascontiguousarray(px, dtype=np.uint8)
        if buf.size != w * h * ncomp:
            raise InvalidInput("pixel buffer length does not match the image dimensions")
        out = _u8p()
        n = ctypes.c_size_t()
        with self._lock:
            rc = self.lib.jp2g_encode(self.handle, buf.ctypes.data_as(ctypes.c_void_p), w, h, ncomp,
                                      int(interleaved), quality, fmt, ctypes.byref(out), ctypes.byref(n))
            self._check(rc)
        data = ctypes.string_at(out, n.value)
        self.lib.jp2g_free(out)
        return data

    def encode_with_psnr(self, px, w: int, h: int, ncomp: int, quality: int, fmt: int,
                         interleaved: bool = True):
        """(codestream, psnr_db, ssim): the encode and its quality metrics,
        computed on the device (encode_with_psnr, src/encode/mod.rs:129)."""
        buf = np.frombuffer(px, dtype=np.uint8) if isinstance(px, (bytes, bytearray)) else \
            np.ascontiguousarray(px, dtype=np.uint8)
        if buf.size != w * h * ncomp:
            raise InvalidInput("pixel buffer length does not match the image dimensions")
        out = _u8p()
        n = ctypes.c_size_t()
        psnr, ssim = ctypes.c_double(), ctypes.c_double()
        with self._lock:
            rc = self.lib.jp2g_encode_with_psnr(self.handle, buf.ctypes.data_as(ctypes.c_void_p), w, h, ncomp,
                                                int(interleaved), quality, fmt, ctypes.byref(out), ctypes.byref(n),
                                                ctypes.byref(psnr), ctypes.byref(ssim))
            self._check(rc)
        data = ctypes.string_at(out, n.value)
        self.lib.jp2g_free(out)
        return data, psnr.value, ssim.value

    @staticmethod
    def _decode_flags(rct_chroma_extra_bitplane, accept_empty_segments):
        return (1 if rct_chroma_extra_bitplane else 0) | (2 if accept_empty_segments else 0)

    def decode(self, data: bytes, rct_chroma_extra_bitplane: bool = False, accept_empty_segments: bool = False):
        """(pixels, w, h, ncomp): a J2K/JP2 file decoded on the device
        (decode_jp2, src/decode/mod.rs:56-61); pixels interleaved, as a uint8
        array over the library's buffer. The two options relax the reference
        decoder's checks (include/jp2g.h)."""
        buf = np.frombuffer(bytes(data), dtype=np.uint8)
        out = _u8p()
        n = ctypes.c_size_t()
        w, h, c = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        with self._lock:
            rc = self.lib.jp2g_decode(self.handle, buf.ctypes.data_as(ctypes.c_void_p), buf.size,
                                      self._decode_flags(rct_chroma_extra_bitplane, accept_empty_segments),
                                      ctypes.byref(out), ctypes.byref(n),
                                      ctypes.byref(w), ctypes.byref(h), ctypes.byref(c))
            self._check(rc)
        return self._owned(out, n.value), w.value, h.value, c.value

    def decode_batch(self, files, rct_chroma_extra_bitplane: bool = False, accept_empty_segments: bool = False):
        """jp2g_decode_batch: a list with, per file, (pixels, w, h, ncomp) or
        the Jp2LamError it failed with; pixels as in decode."""
        n = len(files)
        if n == 0:
            return []
        keep = [np.frombuffer(bytes(f), dtype=np.uint8) for f in files]
        ptrs = (ctypes.c_void_p * n)(*[k.ctypes.data for k in keep])
        lens = (ctypes.c_size_t * n)(*[k.size for k in keep])
        outs = (ctypes.c_void_p * n)()
        out_lens = (ctypes.c_size_t * n)()
        ws, hs, cs = (ctypes.c_uint32 * n)(), (ctypes.c_uint32 * n)(), (ctypes.c_uint32 * n)()
        status = (ctypes.c_int * n)()
        with self._lock:
            self.lib.jp2g_decode_batch(self.handle, ptrs, lens, n,
                                       self._decode_flags(rct_chroma_extra_bitplane, accept_empty_segments), outs,
                                       out_lens, ws, hs, cs, status)
            msg = self.lib.jp2g_last_error(self.handle)
            msg = msg.decode() if isinstance(msg, bytes) else str(msg)
        res = []
        for i in range(n):
            if status[i] == 0:
                res.append((self._owned(ctypes.cast(outs[i], _u8p), out_lens[i]), ws[i], hs[i], cs[i]))
            else:
                res.append(_BY_CODE.get(status[i], EncodeFailed)(msg))
        return res

    def _owned(self, ptr, n: int) -> np.ndarray:
        """A uint8 array over a buffer the library returned, without a copy;
        the buffer goes back to jp2g_free when the array is collected."""
        if n == 0:
            self.lib.jp2g_free(ptr)
            return np.zeros(0, np.uint8)
        arr = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_uint8)), shape=(n,))
        weakref.finalize(arr, self.lib.jp2g_free, ptr)
        return arr

    def encode_device(self, dev_ptr: int, w: int, h: int, ncomp: int, quality: int, fmt: int) -> bytes:
        out = _u8p()
        n = ctypes.c_size_t()
        with self._lock:
            rc = self.lib.jp2g_encode_device(self.handle, ctypes.c_void_p(dev_ptr), w, h, ncomp, quality,
                                             fmt, ctypes.byref(out), ctypes.byref(n))
            self._check(rc)
        data = ctypes.string_at(out, n.value)
        self.lib.jp2g_free(out)
        return data

    @staticmethod
    def _request(page, keep):
        """Builds a Request from a dict with px (host array/bytes or device
        pointer int with on_device=True), w, h, ncomp, quality, fmt and
        optionally interleaved."""
        on_dev = bool(page.get("on_device", False))
        w, h, nc = int(page["w"]), int(page["h"]), int(page["ncomp"])
        if on_dev:
            ptr = int(page["px"])
        else:
            px = page["px"]
            buf = np.frombuffer(px, dtype=np.uint8) if isinstance(px, (bytes, bytearray)) else \
                np.ascontiguousarray(px, dtype=np.uint8)
            if buf.size != w * h * nc:
                raise InvalidInput("pixel buffer length does not match the image dimensions")
            keep.append(buf)
            ptr = buf.ctypes.data
        return Request(ptr, w, h, nc, int(page.get("interleaved", True)), int(on_dev),
                       int(page["quality"]), int(page["fmt"]))

    def encode_batch(self, pages):
        """Encodes a list of page dicts in device waves. Returns a list with
        the codestream bytes of each page, or the exception its status maps
        to."""
        keep = []
        n = len(pages)
        reqs = (Request * max(n, 1))(*[self._request(p, keep) for p in pages])
        outs = (_u8p * max(n, 1))()
        lens = (ctypes.c_size_t * max(n, 1))()
        status = (ctypes.c_int * max(n, 1))()
        with self._lock:
            rc = self.lib.jp2g_encode_batch(self.handle, reqs, n, outs, lens, status)
            msg = self.lib.jp2g_last_error(self.handle).decode() if rc != 0 else ""
        result = []
        for i in range(n):
            if status[i] == 0:
                result.append(ctypes.string_at(outs[i], lens[i]))
                self.lib.jp2g_free(outs[i])
            else:
                result.append(_BY_CODE.get(status[i], Jp2LamError)(msg or f"page {i} failed"))
        return result

    def submit(self, page) -> int:
        """Queues one page dict for continuous batching; returns its ticket."""
        keep = []
        req = self._request(page, keep)
        t = ctypes.c_uint64()
        rc = self.lib.jp2g_submit(self.handle, ctypes.byref(req), ctypes.byref(t))
        self._check(rc)
        with self._inflight_lock:
            self._inflight[t.value] = keep
        return t.value

    def poll(self, ticket: int, timeout_ms: int = -1):
        """The ticket's codestream, or None if it is not done within
        timeout_ms. Raises the page's error if it failed."""
        out = _u8p()
        n = ctypes.c_size_t()
        rc = self.lib.jp2g_poll(self.handle, ticket, ctypes.byref(out), ctypes.byref(n), timeout_ms)
        if rc == PENDING:
            return None
        with self._inflight_lock:
            self._inflight.pop(ticket, None)
        self._check(rc)
        data = ctypes.string_at(out, n.value)
        self.lib.jp2g_free(out)
        return data

    def cancel(self, ticket: int) -> bool:
        """Cancels a submitted page. True: it never reached the device, or
        it had finished and its result is dropped; its ticket and pixels are
        released. False: its wave is in flight, its result is dropped and
        poll() raises EncodeFailed once the wave is done."""
        rc = self.lib.jp2g_cancel(self.handle, ticket)
        if rc == PENDING:
            return False
        self._check(rc)
        with self._inflight_lock:
            self._inflight.pop(ticket, None)
        return True

    def debug_assemble_device(self, w: int, h: int, ncomp: int, quality: int, fmt: int, npasses, zbp, seg_len,
                              body) -> bytes:
        """Device Tier-2 alone on the inputs of debug_assemble()."""
        npasses = np.ascontiguousarray(npasses, dtype=np.uint16)
        zbp = np.ascontiguousarray(zbp, dtype=np.uint8)
        seg_len = np.ascontiguousarray(seg_len, dtype=np.uint32)
        body = np.ascontiguousarray(np.frombuffer(bytes(body), np.uint8) if not isinstance(body, np.ndarray)
                                    else body, dtype=np.uint8)
        out = _u8p()
        n = ctypes.c_size_t()
        ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        with self._lock:
            rc = self.lib.jp2g_debug_assemble_device(self.handle, w, h, ncomp, quality, fmt, ptr(npasses), ptr(zbp),
                                                     ptr(seg_len), ptr(body) if body.size else None, len(npasses),
                                                     ctypes.byref(out), ctypes.byref(n))
            self._check(rc)
        data = ctypes.string_at(out, n.value)
        self.lib.jp2g_free(out)
        return data

    def set_option(self, option: int, value: int):
        self._check(self.lib.jp2g_set_option(self.handle, option, value))

    def get_option(self, option: int) -> int:
        v = ctypes.c_int64()
        self._check(self.lib.jp2g_get_option(self.handle, option, ctypes.byref(v)))
        return v.value

    def autotune(self, pages, repeats: int = 2):
        """Picks the fastest MQ schedule and wave size for a sample of page
        dicts (as encode_batch takes them) and leaves it set; returns
        ({option: value}, wall ms of one encode of the sample)."""
        keep = []
        n = len(pages)
        reqs = (Request * max(n, 1))(*[self._request(p, keep) for p in pages])
        best = (ctypes.c_int64 * NUM_OPTS)()
        ms = ctypes.c_double()
        with self._lock:
            rc = self.lib.jp2g_autotune(self.handle, reqs, n, repeats, best, ctypes.byref(ms))
            msg = self.lib.jp2g_last_error(self.handle).decode() if rc != 0 else ""
        if rc != 0:
            raise _BY_CODE.get(rc, Jp2LamError)(msg)
        return {i: best[i] for i in range(NUM_OPTS)}, ms.value

    def stream(self) -> int:
        return self.lib.jp2g_stream(self.handle)

    def set_timing(self, on: bool):
        self.lib.jp2g_set_timing(self.handle, int(on))

    def stage_times(self):
        ms = (ctypes.c_float * 12)()
        self.lib.jp2g_stage_times(self.handle, ms, 12)
        keys = ["h2d", "dwt", "tier1", "pcrd", "compact", "d2h", "host", "total",
                "t1_analyze", "t1_model", "t1_mq", "tier2"]
        return dict(zip(keys, list(ms)))

    def counters(self):
        c = (ctypes.c_uint64 * 8)()
        self.lib.jp2g_counters(self.handle, c, 8)
        return list(c)

    def debug_coefficients(self, px, w, h, ncomp, quality, comp):
        px = np.ascontiguousarray(px, dtype=np.uint8)
        plane = np.zeros(w * h, np.int32)
        self._check(self.lib.jp2g_debug_coefficients(self.handle, px.ctypes.data_as(ctypes.c_void_p), w, h,
                                                     ncomp, quality, comp,
                                                     plane.ctypes.data_as(ctypes.c_void_p)))
        return plane.reshape(h, w)

    def debug_coefficients_f32(self, px, w, h, ncomp, quality, comp):
        """Unquantised f32 coefficients (lossy qualities) of one component."""
        px = np.ascontiguousarray(px, dtype=np.uint8)
        out = np.zeros(w * h, np.float32)
        self._check(self.lib.jp2g_debug_coefficients_f32(self.handle, px.ctypes.data_as(ctypes.c_void_p), w, h,
                                                         ncomp, quality, comp, out.ctypes.data_as(ctypes.c_void_p)))
        return out.reshape(h, w)

    def debug_blocks(self, px, w, h, ncomp, quality):
        px = np.ascontiguousarray(px, dtype=np.uint8)
        n = ctypes.c_uint32()
        self._check(self.lib.jp2g_debug_blocks(self.handle, px.ctypes.data_as(ctypes.c_void_p), w, h, ncomp,
                                               quality, None, 0, ctypes.byref(n)))
        rows = np.zeros(8 * n.value, np.int32)
        self._check(self.lib.jp2g_debug_blocks(self.handle, px.ctypes.data_as(ctypes.c_void_p), w, h, ncomp,
                                               quality, rows.ctypes.data_as(ctypes.c_void_p), n.value,
                                               ctypes.byref(n)))
        return rows.reshape(-1, 8)


def context_labels():
    """The bit-sliced context formation evaluated on single samples, in the
    layout of tables() (zc, sc, spb)."""
    lib = load_library()
    zc = np.zeros(2048, np.uint8)
    sc = np.zeros(256, np.uint8)
    spb = np.zeros(256, np.uint8)
    lib.jp2g_debug_context_labels(*(a.ctypes.data_as(ctypes.c_void_p) for a in (zc, sc, spb)))
    return zc, sc, spb


def tables():
    """The Tier-1/MQ tables the kernels use (host-only, no GPU needed)."""
    lib = load_library()
    zc = np.zeros(2048, np.uint8)
    sc = np.zeros(256, np.uint8)
    spb = np.zeros(256, np.uint8)
    mq = np.zeros(94, np.uint32)
    lib.jp2g_tables(*(a.ctypes.data_as(ctypes.c_void_p) for a in (zc, sc, spb, mq)))
    return zc, sc, spb, mq


def debug_assemble(w: int, h: int, ncomp: int, quality: int, fmt: int, npasses, zbp, seg_len,
                   body) -> bytes:
    """Host Tier-2 alone (host-only, no GPU needed): the codestream of a page
    whose code-blocks, in codestream order, retain npasses[i] passes in one
    segment of seg_len[i] bytes (consecutive in body) above zbp[i] zero
    bit-planes."""
    lib = load_library()
    npasses = np.ascontiguousarray(npasses, dtype=np.uint16)
    zbp = np.ascontiguousarray(zbp, dtype=np.uint8)
    seg_len = np.ascontiguousarray(seg_len, dtype=np.uint32)
    body = np.ascontiguousarray(np.frombuffer(bytes(body), np.uint8) if not isinstance(body, np.ndarray) else body,
                                dtype=np.uint8)
    out = _u8p()
    n = ctypes.c_size_t()
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    rc = lib.jp2g_debug_assemble(w, h, ncomp, quality, fmt, ptr(npasses), ptr(zbp), ptr(seg_len),
                                 ptr(body) if body.size else None, len(npasses), ctypes.byref(out),
                                 ctypes.byref(n))
    if rc != 0:
        _raise(rc, "host Tier-2 assembly failed")
    data = ctypes.string_at(out, n.value)
    lib.jp2g_free(out)
    return data


def debug_plan(w: int, h: int, ncomp: int, quality: int) -> dict:
    """The encoding plan (host-only, no GPU needed): levels, code-block
    width, quantiser entries (res, band, exponent, mantissa), code-blocks and
    the PCRD lambdas at the quality and at 1."""
    lib = load_library()
    lv, cbw, nq, nb = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_uint32()
    q = np.zeros(4 * 32, np.int32)
    lam = np.zeros(2, np.float64)
    rc = lib.jp2g_debug_plan(w, h, ncomp, quality, ctypes.byref(lv), ctypes.byref(cbw), ctypes.byref(nq),
                             q.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nb), lam.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        _raise(rc, "plan failed")
    return {"levels": lv.value, "cbw": cbw.value, "quants": [tuple(q[4 * i:4 * i + 4]) for i in range(nq.value)],
            "nblocks": nb.value, "lambdas": (float(lam[0]), float(lam[1]))}


_default = None


def default_engine() -> Engine:
    global _default
    with _engine_lock:
        if _default is None:
            _default = Engine(0)
        return _default


# ------------------------------------------------------------- synthetic ----
_synth = None


def synth_page(w: int, h: int, ncomp: int, seed: int, glyphs: int = -1, photo_w: int = 0,
               photo_h: int = 0, photo_frac: float = 0.0) -> np.ndarray:
    """Seeded synthetic document page, interleaved uint8 (h, w, ncomp)."""
    global _synth
    if _synth is None:
        if not os.path.exists(SYNTH_PATH):
            from . import build as _b
            _b.build_synth()
        _synth = ctypes.CDLL(SYNTH_PATH)
        _synth.jp2g_synth_page.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                           ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_double]
    out = np.zeros(w * h * ncomp, np.uint8)
    rc = _synth.jp2g_synth_page(out.ctypes.data_as(ctypes.c_void_p), w, h, ncomp, ctypes.c_uint64(seed),
                                glyphs, photo_w, photo_h, photo_frac)
    if rc < 0:
        raise InvalidInput("bad synthetic page parameters")
    return out
