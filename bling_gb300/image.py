"""Image output of a rendered film: the step after film accumulation.

The reference turns its film into pixels with ``getPixel`` (XYZ / weight,
then ``xyzToRgb``; ``Image.hs:302-315``) and writes them as PNG or Radiance
HDR through JuicyPixels (``IO/Bitmap.hs:31-41``); its 8-bit path applies
``gamma 2.2`` and ``clamp`` (``Image.hs:318-331``).  Here the film is
resolved to linear RGB by ``bling_film_resolve`` (``Film.resolve()``) or
:func:`resolve` below, and these functions do the rest on the host:

* :func:`to_rgb8` -- ``rgbPixels``: gamma 2.2, clamp to [0, 1], scale to
  0..255 and round half to even (Haskell's ``round``);
* :func:`write_png` -- an 8-bit RGB PNG (zlib-compressed scanlines, filter
  type 0);
* :func:`write_rgbe` -- a Radiance ``.hdr`` file with flat (uncompressed)
  RGBE scanlines, the shared-exponent encoding of the Radiance format.

The encoders are written from the published file formats (PNG: RFC 2083;
Radiance RGBE: Ward, "Real Pixels", Graphics Gems II).
"""
from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np

F = np.float32


def resolve(film: np.ndarray, splats: np.ndarray | None = None,
            splat_weight: float = 0.0) -> np.ndarray:
    """(h, w, 4) film (weight, X, Y, Z) -> (h, w, 3) linear RGB, float32:
    getPixel (Image.hs:302-315) and xyzToRgb (Spectrum.hs:162-168), in the
    reference's binary32 order.  splats: the (h, w, 3) XYZ splat image of
    light passes, added with splat_weight (1 / (passes * photons per pass)
    for the light tracer, LightTracer.hs:44)."""
    from .spectrum import xyz_to_rgb
    f = np.asarray(film, np.float32)
    w = f[..., 0]
    inv = np.where(w != 0, F(1) / np.where(w != 0, w, F(1)), F(0)).astype(np.float32)
    x, y, z = f[..., 1] * inv, f[..., 2] * inv, f[..., 3] * inv
    if splats is not None:
        sw = F(splat_weight)
        sp = np.asarray(splats, np.float32)
        x, y, z = sw * sp[..., 0] + x, sw * sp[..., 1] + y, sw * sp[..., 2] + z
    r, g, b = xyz_to_rgb(x, y, z)
    return np.stack([r, g, b], -1).astype(np.float32)


def to_rgb8(rgb: np.ndarray, gamma: float = 2.2) -> np.ndarray:
    """rgbPixels' per-pixel mapping (Image.hs:318-331): v ** (1/gamma), then
    round(min 1 (max 0 v) * 255) with round half to even."""
    v = np.asarray(rgb, np.float32)
    ig = F(1) / F(gamma)
    # NaN and negative values clamp to 0 before the power (x ** y of a
    # negative base is NaN, which max 0 turns into 0 in the reference too)
    v = np.power(np.maximum(v, F(0)), ig, dtype=np.float32)
    v = np.minimum(F(1), np.maximum(F(0), np.nan_to_num(v, nan=0.0)))
    return np.rint(v * F(255)).astype(np.uint8)


def _png_chunk(kind: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data))


def write_png(path: str | Path, rgb8: np.ndarray) -> None:
    """An 8-bit truecolour PNG of an (h, w, 3) uint8 array."""
    a = np.ascontiguousarray(rgb8, np.uint8)
    if a.ndim != 3 or a.shape[2] != 3:
        raise ValueError("expected an (h, w, 3) uint8 image")
    h, w, _ = a.shape
    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(h))  # filter 0 per scanline
    png = (b"\x89PNG\r\n\x1a\n"
           + _png_chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
           + _png_chunk(b"IDAT", zlib.compress(raw, 6))
           + _png_chunk(b"IEND", b""))
    Path(path).write_bytes(png)


def _paeth(a: int, b: int, c: int) -> int:
    """the Paeth predictor (PNG specification, filter type 4)"""
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def read_png(path: str | Path) -> np.ndarray:
    """Reads an 8-bit, non-interlaced PNG (RFC 2083): grey (h, w), grey with
    alpha (h, w, 2), RGB (h, w, 3), RGBA (h, w, 4), or a palette image as RGB.
    Every scanline filter (none, sub, up, average, Paeth) is undone."""
    data = Path(path).read_bytes()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, w, h, ctype, palette = 8, b"", 0, 0, 0, None
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body[:13])
            if depth != 8 or interlace != 0 or ctype not in (0, 2, 3, 4, 6):
                raise ValueError("only 8-bit, non-interlaced PNGs are read")
        elif kind == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"IDAT":
            idat += body
        elif kind == b"IEND":
            break
        pos += 12 + n
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    stride = w * ch
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + stride)
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        ft, line = raw[y, 0], raw[y, 1:].astype(np.int32)
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 255
        else:  # sub, average and Paeth read the reconstructed bytes to the left
            cur = np.zeros(stride, np.int32)
            for i in range(stride):
                left = cur[i - ch] if i >= ch else 0
                if ft == 1:
                    pred = left
                elif ft == 3:
                    pred = (left + prev[i]) >> 1
                elif ft == 4:
                    pred = _paeth(left, prev[i], prev[i - ch] if i >= ch else 0)
                else:
                    raise ValueError(f"unknown PNG filter type {ft}")
                cur[i] = (line[i] + pred) & 255
        out[y] = cur
        prev = cur
    img = out.reshape(h, w, ch)
    if ctype == 3:
        if palette is None:
            raise ValueError("palette PNG without PLTE")
        return palette[img[..., 0]].copy()
    return img[..., 0].copy() if ch == 1 else img.copy()


def rgbe_encode(rgb: np.ndarray) -> np.ndarray:
    """(…, 3) linear RGB -> (…, 4) uint8 RGBE: mantissas scaled by 2^-e with e
    the exponent of the largest component (frexp), 0 0 0 0 below 1e-32."""
    v = np.maximum(np.asarray(rgb, np.float64), 0.0)
    m = v.max(-1)
    mant, e = np.frexp(m)
    scale = np.where(m > 1e-32, mant * 256.0 / np.where(m > 1e-32, m, 1.0), 0.0)
    out = np.zeros(v.shape[:-1] + (4,), np.uint8)
    out[..., :3] = np.clip(np.floor(v * scale[..., None]), 0, 255).astype(np.uint8)
    out[..., 3] = np.where(m > 1e-32, e + 128, 0).astype(np.uint8)
    return out


def rgbe_decode(rgbe: np.ndarray) -> np.ndarray:
    """(…, 4) uint8 RGBE -> (…, 3) float32 (the value at the middle of each
    mantissa step)."""
    q = np.asarray(rgbe)
    e = q[..., 3].astype(np.int32)
    f = np.where(e > 0, np.ldexp(1.0, e - (128 + 8)), 0.0)
    return ((q[..., :3].astype(np.float64) + 0.5) * f[..., None]).astype(np.float32)


def write_rgbe(path: str | Path, rgb: np.ndarray) -> None:
    """A Radiance .hdr file of an (h, w, 3) linear RGB image, flat scanlines."""
    a = np.asarray(rgb, np.float32)
    h, w, _ = a.shape
    head = f"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y {h} +X {w}\n".encode("ascii")
    Path(path).write_bytes(head + rgbe_encode(a).tobytes())


def read_rgbe(path: str | Path) -> np.ndarray:
    """Reads back a flat-scanline Radiance .hdr file (as write_rgbe writes)."""
    data = Path(path).read_bytes()
    end = data.index(b"\n\n") + 2
    line_end = data.index(b"\n", end)
    dims = data[end:line_end].decode("ascii").split()
    h, w = int(dims[1]), int(dims[3])
    q = np.frombuffer(data[line_end + 1:line_end + 1 + 4 * w * h], np.uint8).reshape(h, w, 4)
    return rgbe_decode(q)
