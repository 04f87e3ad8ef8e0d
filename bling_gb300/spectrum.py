"""16-band spectra for scene description (host side, binary32).

The band tables are the generated ``csrc/spectrum_tables.h`` (derived from
bling's Spectrum.hs by ``gen_spectrum_tables.py``); this module reads the bit
patterns from that header so the host and the GPU use identical values.
"""
from __future__ import annotations

import re
from functools import lru_cache
from pathlib import Path

import numpy as np

F = np.float32
_HDR = Path(__file__).with_name("csrc") / "spectrum_tables.h"
BASES = ["white", "cyan", "magenta", "yellow", "red", "green", "blue"]


@lru_cache(maxsize=None)
def tables() -> dict:
    src = _HDR.read_text()
    out = {}
    for m in re.finditer(r"static const uint32_t (\w+)\[(\d+)\] = \{(.*?)\};", src, re.S):
        vals = [int(x, 16) for x in re.findall(r"0x([0-9a-f]{8})u", m.group(3))]
        out[m.group(1)] = np.asarray(vals, dtype=np.uint32).view(np.float32)
    ysum = int(re.search(r"BLING_CIE_Y_SUM_BITS 0x([0-9a-f]{8})u", src).group(1), 16)
    out["Y_SUM"] = np.asarray([ysum], dtype=np.uint32).view(np.float32)[0]
    return out


def _basis(illum: bool, name: str) -> np.ndarray:
    t = tables()["BLING_RGB_ILLUM_BITS" if illum else "BLING_RGB_REFL_BITS"]
    k = BASES.index(name)
    return t[16 * k:16 * (k + 1)]


def rgb_to_spectrum(rgb, illuminant: bool = False) -> np.ndarray:
    """rgbToSpectrumRefl / rgbToSpectrumIllum (Spectrum.hs:140-159)."""
    r, g, b = (F(x) for x in rgb)

    def sc(name, f):
        return (_basis(illuminant, name) * F(f)).astype(np.float32)

    if r <= g and r <= b:
        rest = sc("cyan", g - r) + sc("blue", b - g) if g <= b else sc("cyan", b - r) + sc("green", g - b)
        return (sc("white", r) + rest).astype(np.float32)
    if g <= r and g <= b:
        rest = sc("magenta", r - g) + sc("blue", b - r) if r <= b else sc("magenta", b - g) + sc("red", r - b)
        return (sc("white", g) + rest).astype(np.float32)
    rest = sc("yellow", r - b) + sc("green", g - r) if r <= b else sc("yellow", g - b) + sc("red", r - g)
    return (sc("white", b) + rest).astype(np.float32)


def rgb_to_spectrum_array(rgb, illuminant: bool = False) -> np.ndarray:
    """rgb_to_spectrum for an (..., 3) array; per element the same binary32
    operations as the scalar version."""
    rgb = np.asarray(rgb, dtype=np.float32)
    r, g, b = (rgb[..., k][..., None] for k in range(3))
    B = {n: _basis(illuminant, n) for n in BASES}

    def sc(name, f):
        return (B[name] * f).astype(np.float32)

    c1 = (sc("white", r) + np.where(g <= b, sc("cyan", g - r) + sc("blue", b - g),
                                    sc("cyan", b - r) + sc("green", g - b))).astype(np.float32)
    c2 = (sc("white", g) + np.where(r <= b, sc("magenta", r - g) + sc("blue", b - r),
                                    sc("magenta", b - g) + sc("red", r - b))).astype(np.float32)
    c3 = (sc("white", b) + np.where(r <= b, sc("yellow", r - b) + sc("green", g - r),
                                    sc("yellow", g - b) + sc("red", r - g))).astype(np.float32)
    case1 = (r <= g) & (r <= b)
    case2 = (g <= r) & (g <= b)
    return np.where(case1, c1, np.where(case2, c2, c3)).astype(np.float32)


def constant(v: float) -> np.ndarray:
    return np.full(16, F(v), dtype=np.float32)


def spectrum_to_xyz(s) -> tuple:
    """spectrumToXYZ (Spectrum.hs:349-355), sequential binary32 sums."""
    t = tables()
    a = b = c = F(0)
    for i in range(16):
        v = F(s[i])
        a = a + t["BLING_CIE_X_BITS"][i] * v
        b = b + t["BLING_CIE_Y_BITS"][i] * v
        c = c + t["BLING_CIE_Z_BITS"][i] * v
    ys = t["Y_SUM"]
    return a / ys, b / ys, c / ys


def xyz_to_rgb(x, y, z):
    """xyzToRgb (Spectrum.hs:162-168), vectorised over arrays."""
    x, y, z = (np.asarray(v, dtype=np.float32) for v in (x, y, z))
    r = F(3.240479) * x - F(1.537150) * y - F(0.498535) * z
    g = F(-0.969256) * x + F(1.875991) * y + F(0.041556) * z
    b = F(0.055648) * x - F(0.204043) * y + F(1.057311) * z
    return r, g, b
