"""jp2lam_gb300 — GB300-native JPEG 2000 encoder with jp2lam's encode API.

Python mirror of the reference's public encode surface (src/lib.rs:19-29),
backed by the C ABI in include/jp2g.h (libjp2g.so, CUDA for sm_103a):

    Image.from_gray_bytes / Image.from_rgb_bytes   (src/model.rs:87-140)
    EncodeOptions(quality, format), Preset          (src/model.rs:41-177)
    encode(image, options) -> bytes                 (src/encode/mod.rs:84-101)
    encode_to_writer(image, options, writer)        (src/encode/mod.rs:103-113)
    encode_with_psnr(image, options)                (src/encode/mod.rs:115-135)
    BatchEncoder(options).encode_one / encode_all   (src/batch.rs:26-85)
    encode_batch(images, options)                   (src/batch.rs:173-178)
    decode_jp2(bytes) -> Image                      (src/decode/mod.rs:56-61)

Errors are Jp2LamError subclasses carrying the reference's variant names.
The compute path is the CUDA library only; if it cannot be loaded or no GPU
is present, encoding raises instead of falling back to the CPU.
"""
from __future__ import annotations

import enum
from dataclasses import dataclass, field
from typing import Iterable, List, Optional

from ._native import Engine, Jp2LamError, InvalidInput, EncodeFailed, DecodeFailed, \
    UnsupportedFeature, IoError, default_engine

__all__ = [
    "ColorSpace", "OutputFormat", "Preset", "Image", "Component", "EncodeOptions",
    "encode", "encode_to_writer", "encode_with_psnr", "EncodeMetrics", "BatchEncoder", "BatchProfile", "encode_batch",
    "encode_pages", "decode_jp2", "decode_batch", "Server", "Engine", "Jp2LamError", "InvalidInput", "EncodeFailed", "DecodeFailed",
    "UnsupportedFeature", "IoError",
]


class ColorSpace(enum.Enum):
    GRAY = "Gray"
    SRGB = "Srgb"

    def component_count(self) -> int:
        return 1 if self is ColorSpace.GRAY else 3


class OutputFormat(enum.IntEnum):
    J2K = 0
    JP2 = 1


class Preset(enum.Enum):
    """src/model.rs:41-62"""
    DOCUMENT_LOW = 30
    DOCUMENT_HIGH = 85
    WEB_LOW = 42
    WEB_HIGH = 62

    def quality(self) -> int:
        return self.value


@dataclass
class Component:
    width: int
    height: int
    precision: int = 8
    signed: bool = False
    dx: int = 1
    dy: int = 1


@dataclass
class Image:
    """Interleaved 8-bit pixels plus the reference Image's metadata."""
    width: int
    height: int
    colorspace: ColorSpace
    data: bytes
    components: List[Component] = field(default_factory=list)

    @staticmethod
    def from_gray_bytes(width: int, height: int, data) -> "Image":
        data = bytes(data)
        expected = width * height
        if len(data) != expected:
            raise InvalidInput(
                f"Gray buffer length {len(data)} does not match {width}×{height}={expected}")
        return Image(width, height, ColorSpace.GRAY, data, [Component(width, height)])

    @staticmethod
    def from_rgb_bytes(width: int, height: int, data) -> "Image":
        data = bytes(data)
        expected = width * height * 3
        if len(data) != expected:
            raise InvalidInput(
                f"RGB buffer length {len(data)} does not match {width}×{height}×3={expected}")
        return Image(width, height, ColorSpace.SRGB, data, [Component(width, height) for _ in range(3)])

    @property
    def ncomp(self) -> int:
        return self.colorspace.component_count()


@dataclass
class EncodeOptions:
    """src/model.rs:156-177 (default: DocumentHigh quality, JP2)."""
    quality: int = 85
    format: OutputFormat = OutputFormat.JP2

    @staticmethod
    def from_preset(preset: Preset, fmt: OutputFormat) -> "EncodeOptions":
        return EncodeOptions(preset.quality(), fmt)


def _validate(image: Image) -> None:
    # validate_image (src/plan/validate.rs:4-62)
    if image.width == 0 or image.height == 0:
        raise InvalidInput("image dimensions must be non-zero")
    if len(image.components) != image.colorspace.component_count():
        raise InvalidInput(f"{image.colorspace.value} images must have exactly "
                           f"{image.colorspace.component_count()} component(s)")
    for idx, c in enumerate(image.components):
        if c.width != image.width or c.height != image.height:
            raise InvalidInput(f"component {idx} dimensions {c.width}x{c.height} do not match "
                               f"image {image.width}x{image.height}")
        if c.precision != 8:
            raise InvalidInput(f"component {idx} precision {c.precision} is unsupported; "
                               "only 8-bit is supported")
        if c.signed:
            raise InvalidInput(f"component {idx} must be unsigned")
        if c.dx != 1 or c.dy != 1:
            raise InvalidInput(f"component {idx} subsampling {c.dx}x{c.dy} is unsupported")
    if len(image.data) != image.width * image.height * image.ncomp:
        raise InvalidInput("pixel buffer length does not match the image dimensions")


def encode(image: Image, options: Optional[EncodeOptions] = None,
           engine: Optional[Engine] = None) -> bytes:
    """Encode one page on the GPU; byte-identical to jp2lam::encode."""
    options = options or EncodeOptions()
    _validate(image)
    eng = engine or default_engine()
    return eng.encode(image.data, image.width, image.height, image.ncomp,
                      int(options.quality), int(options.format))


def encode_to_writer(image: Image, options: EncodeOptions, writer) -> None:
    data = encode(image, options)
    try:
        writer.write(data)
    except Exception as err:  # mirrors EncodeFailed(err.to_string())
        raise EncodeFailed(str(err)) from err


@dataclass(frozen=True)
class EncodeMetrics:
    """src/encode/mod.rs:115-123: PSNR in dB (+inf for lossless) and the
    mean SSIM of 8x8 luma blocks (1.0 for lossless)."""
    psnr_db: float
    ssim: float


def encode_with_psnr(image: Image, options: EncodeOptions,
                     engine: Optional[Engine] = None):
    """Encode and compute the quality metrics in one call
    (src/encode/mod.rs:129-135); the decoder-side reconstruction behind the
    metrics runs on the GPU. Returns (bytes, EncodeMetrics)."""
    _validate(image)
    eng = engine or default_engine()
    data, psnr, ssim = eng.encode_with_psnr(image.data, image.width, image.height, image.ncomp,
                                            int(options.quality), int(options.format))
    return data, EncodeMetrics(psnr, ssim)


def decode_jp2(data: bytes, engine: Optional[Engine] = None,
               rct_chroma_extra_bitplane: bool = False, accept_empty_segments: bool = False) -> Image:
    """Decode a J2K/JP2 file of this encoder's profile on the GPU
    (decode_jp2, src/decode/mod.rs:56-61). rct_chroma_extra_bitplane counts
    the extra chroma bit-plane that lossless sRGB encodes use and QCD does not
    signal; accept_empty_segments decodes code-blocks that have passes but no
    bytes. Without them such files fail as they do in the reference."""
    eng = engine or default_engine()
    px, w, h, c = eng.decode(data, rct_chroma_extra_bitplane, accept_empty_segments)
    if c == 1:
        return Image.from_gray_bytes(w, h, px)
    return Image.from_rgb_bytes(w, h, px)


def decode_batch(files, engine: Optional[Engine] = None, rct_chroma_extra_bitplane: bool = False,
                 accept_empty_segments: bool = False):
    """decode_jp2 over many files in shared device launches: per file an
    Image, or the Jp2LamError it failed with."""
    eng = engine or default_engine()
    out = []
    for r in eng.decode_batch(files, rct_chroma_extra_bitplane, accept_empty_segments):
        if isinstance(r, Jp2LamError):
            out.append(r)
        else:
            px, w, h, c = r
            out.append(Image.from_gray_bytes(w, h, px) if c == 1 else Image.from_rgb_bytes(w, h, px))
    return out


@dataclass(frozen=True)
class BatchProfile:
    """src/batch.rs:5-24"""
    width: int
    height: int
    colorspace: ColorSpace
    components: tuple
    quality: int
    format: OutputFormat

    @staticmethod
    def from_image(image: Image, options: EncodeOptions) -> "BatchProfile":
        comps = tuple((c.width, c.height, c.precision, c.signed, c.dx, c.dy) for c in image.components)
        return BatchProfile(image.width, image.height, image.colorspace, comps,
                            int(options.quality), OutputFormat(options.format))


class BatchEncoder:
    """src/batch.rs:26-85: pins the profile of the first image and rejects
    mismatches; every page is encoded on the GPU."""

    def __init__(self, options: Optional[EncodeOptions] = None, engine: Optional[Engine] = None):
        self.options = options or EncodeOptions()
        self._profile: Optional[BatchProfile] = None
        self._count = 0
        self._engine = engine

    def profile(self) -> Optional[BatchProfile]:
        return self._profile

    def encoded_count(self) -> int:
        return self._count

    def _validate_or_set_profile(self, image: Image) -> None:
        prof = BatchProfile.from_image(image, self.options)
        if self._profile is None:
            self._profile = prof
        elif self._profile != prof:
            raise InvalidInput(f"batch item profile mismatch: expected {self._profile}, found {prof}")

    def encode_one(self, image: Image) -> bytes:
        self._validate_or_set_profile(image)
        out = encode(image, self.options, self._engine)
        self._count += 1
        return out

    def encode_all(self, images: Iterable[Image]) -> List[bytes]:
        """Same results as encode_one on each image in turn, but the pages go
        to the device together (jp2g_encode_batch). As in the reference, a
        profile mismatch at item k fails the call after items 0..k-1."""
        images = list(images)
        bad = None
        for k, im in enumerate(images):
            try:
                _validate(im)
                self._validate_or_set_profile(im)
            except Jp2LamError as err:
                bad = (k, err)
                break
        good = images if bad is None else images[:bad[0]]
        outs = encode_pages([(im, self.options) for im in good], self._engine)
        self._count += len(outs)
        if bad is not None:
            raise bad[1]
        return outs


def encode_batch(images: Iterable[Image], options: EncodeOptions) -> List[bytes]:
    return BatchEncoder(options).encode_all(images)


def _page(image: Image, options: EncodeOptions) -> dict:
    return {"px": image.data, "w": image.width, "h": image.height, "ncomp": image.ncomp,
            "quality": int(options.quality), "fmt": int(options.format)}


def encode_pages(items, engine: Optional[Engine] = None) -> List[bytes]:
    """Encodes (Image, EncodeOptions) pairs of any sizes, colours and
    qualities in device waves; each result equals encode(image, options).
    Raises the first failing page's error."""
    items = list(items)
    for im, _ in items:
        _validate(im)
    eng = engine or default_engine()
    outs = eng.encode_batch([_page(im, op) for im, op in items])
    for o in outs:
        if isinstance(o, Exception):
            raise o
    return outs


class Server:
    """Continuous batching over jp2g_submit / jp2g_poll: pages submitted while
    others are on the device join the next device wave."""

    def __init__(self, engine: Optional[Engine] = None):
        self.engine = engine or default_engine()

    def submit(self, image: Image, options: Optional[EncodeOptions] = None) -> int:
        _validate(image)
        return self.engine.submit(_page(image, options or EncodeOptions()))

    def result(self, ticket: int, timeout_ms: int = -1) -> Optional[bytes]:
        """The codestream, or None if not ready within timeout_ms."""
        return self.engine.poll(ticket, timeout_ms)
