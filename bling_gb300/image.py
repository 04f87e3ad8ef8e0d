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


def read_png(path: str | Path) -> np.ndarray:
    """Reads back an 8-bit RGB PNG with filter type 0 (as write_png writes)."""
    data = Path(path).read_bytes()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            if (depth, ctype) != (8, 2):
                raise ValueError("only 8-bit RGB PNGs are read")
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 3 * w)
    if np.any(rows[:, 0] != 0):
        raise ValueError("only filter type 0 is read")
    return rows[:, 1:].reshape(h, w, 3).copy()


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
