"""Derive bling's 16-band spectral tables and write them as a C header.

bling keeps spectra as 16 bands over 400-700 nm (src/lib/Graphics/Bling/Spectrum.hs:33-46).
Its band values are not literals: they are computed at start-up by ``fromSpd``
(Spectrum.hs:329-335) from regularly sampled SPD tables (the Smits RGB basis
spectra at Spectrum.hs:550-773 and the CIE 1931 colour-matching functions at
Spectrum.hs:775-1139) through ``avgSpd`` (Spectrum.hs:297-305).

This script re-runs that derivation in IEEE binary32 arithmetic, one rounding
per operation in the reference's order, so that the resulting band values are
the ones a GHC build of the reference holds in memory:

* decimal literals are rounded exactly once (``fromRational``), here via
  ``fractions.Fraction`` so no double rounding occurs;
* ``lerp t a b = (1 - t) * a + t * b`` (Math.hs:108-110);
* ``avgSpd`` averages the amplitude samples with indices
  ``floor(n * ((l - s0) / (s1 - s0)))`` clamped to ``[0, n]``, summed left to
  right (``V.sum`` is a strict left fold).

It also copies Perlin's noise permutation (``noisePerms``) out of the
``Texture.hs`` beside ``Spectrum.hs``.  It only needs those two files as
text and is run once, in a checkout that has them; the generated header is
committed::

    python bling_gb300/gen_spectrum_tables.py /path/to/bling/src/lib/Graphics/Bling/Spectrum.hs
"""

from __future__ import annotations

import re
import struct
import sys
from fractions import Fraction
from pathlib import Path

import numpy as np

F = np.float32

BANDS = 16
LAMBDA_START = F(400)
LAMBDA_END = F(700)

BASIS_NAMES = [
    "rgbReflWhite", "rgbReflCyan", "rgbReflMagenta", "rgbReflYellow",
    "rgbReflRed", "rgbReflGreen", "rgbReflBlue",
    "rgbIllumWhite", "rgbIllumCyan", "rgbIllumMagenta", "rgbIllumYellow",
    "rgbIllumRed", "rgbIllumGreen", "rgbIllumBlue",
]


def f32_of_decimal(text: str) -> np.float32:
    """Round a decimal literal to the nearest binary32 (ties to even), once."""
    q = Fraction(text)
    if q == 0:
        return F(0.0)
    sign = -1 if q < 0 else 1
    q = abs(q)
    # Find exponent e with 2^e <= q < 2^(e+1).
    e = q.numerator.bit_length() - q.denominator.bit_length()
    if Fraction(2) ** e > q:
        e -= 1
    e = max(e, -126)  # subnormal range shares the minimum exponent
    scale = Fraction(2) ** (23 - e)
    m = q * scale
    mi = m.numerator // m.denominator
    rem = m - mi
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and mi % 2 == 1):
        mi += 1
    val = Fraction(mi) / scale
    return F(sign * float(val))  # exact: val is representable


def lerp(t, a, b):
    return (F(1) - t) * a + t * b


def avg_regular_spd(s0, s1, amps, l0, l1):
    """``avgSpd (RegularSpd s0 s1 amps) l0 l1`` (Spectrum.hs:297-305)."""
    n = len(amps)
    if l1 <= s0:
        return amps[0]
    if l0 >= s1:
        return amps[-1]

    def idx(l):
        x = F(n) * ((l - s0) / (s1 - s0))
        return max(0, min(n, int(np.floor(x))))

    i0, i1 = idx(l0), idx(l1)
    sl = amps[i0:i1 + 1]
    acc = F(0)
    for a in sl:
        acc = acc + a
    return acc / F(len(sl))


def from_spd(s0, s1, amps):
    """``fromSpd`` (Spectrum.hs:329-335) for a regular SPD."""
    out = []
    for i in range(BANDS):
        l0 = lerp(F(i) / F(BANDS), LAMBDA_START, LAMBDA_END)
        l1 = lerp(F(i + 1) / F(BANDS), LAMBDA_START, LAMBDA_END)
        out.append(avg_regular_spd(s0, s1, amps, l0, l1))
    return out


def parse_list(src: str, name: str) -> list[np.float32]:
    m = re.search(r"^" + name + r"\s*=\s*(?:rgbFunc)?\s*\[(.*?)\]", src, re.S | re.M)
    if not m:
        raise SystemExit(f"table {name} not found")
    body = re.sub(r"--[^\n]*", "", m.group(1))
    toks = [t.strip() for t in body.replace("\n", " ").split(",") if t.strip()]
    return [f32_of_decimal(t) for t in toks]


def hexf(x: np.float32) -> str:
    bits = struct.unpack("<I", struct.pack("<f", float(x)))[0]
    return f"__bling_f32(0x{bits:08x}u) /* {float(x)!r} */"


def eval_regular_spd(l0, l1, amps, l):
    """``evalSpd (RegularSpd l0 l1 amps) l`` (Spectrum.hs:271-280)."""
    n = len(amps)
    if l <= l0:
        return amps[0]
    if l >= l1:
        return amps[-1]
    d1 = F(1) / ((l1 - l0) / F(n - 1))
    x = (l - l0) * d1
    b0 = int(np.floor(x))
    b1 = min(b0 + 1, n - 1)
    dx = x - F(b0)
    return (F(1) - dx) * amps[b0] + dx * amps[b1]


def spd_to_xyz(spd, cie):
    """``spdToXYZ`` (Spectrum.hs:318-326): sums over 360..830 nm in steps of
    1 nm, each a left fold from 0, divided by the sum of y-bar"""
    lam = [F(l) for l in range(360, 831)]
    vs = [eval_regular_spd(*spd, l) for l in lam]
    xs = [eval_regular_spd(F(360), F(830), cie["X"], l) for l in lam]
    ys = [eval_regular_spd(F(360), F(830), cie["Y"], l) for l in lam]
    zs = [eval_regular_spd(F(360), F(830), cie["Z"], l) for l in lam]
    yint = F(0)
    for v in ys:
        yint = yint + v
    acc = []
    for cmf in (xs, ys, zs):
        a = F(0)
        for c, v in zip(cmf, vs):
            a = a + c * v
        acc.append(a / yint)
    return acc


def parse_spd(src: str, name: str):
    """``name = mkSpd' l0 l1 [ ... ]``: (l0, l1, amplitudes)"""
    m = re.search(r"^" + name + r"\s*=\s*mkSpd'\s+(\S+)\s+(\S+)\s*\[(.*?)\]", src, re.S | re.M)
    if not m:
        raise SystemExit(f"SPD {name} not found")
    body = re.sub(r"--[^\n]*", "", m.group(3))
    toks = [t.strip() for t in body.replace("\n", " ").split(",") if t.strip()]
    return f32_of_decimal(m.group(1)), f32_of_decimal(m.group(2)), [f32_of_decimal(t) for t in toks]


def main(argv):
    if len(argv) < 2:
        raise SystemExit("usage: gen_spectrum_tables.py <bling's src/lib/Graphics/Bling/Spectrum.hs>"
                         " [output header]")
    src_path = Path(argv[1])
    out_path = Path(argv[2]) if len(argv) > 2 else Path(__file__).with_name("csrc") / "spectrum_tables.h"
    src = src_path.read_text()

    tables = {}
    for name in BASIS_NAMES:
        amps = parse_list(src, name)
        assert len(amps) == 32, (name, len(amps))
        tables[name] = from_spd(F(380), F(720), amps)
    for axis in "XYZ":
        amps = parse_list(src, f"cie{axis}Values")
        assert len(amps) == 471, (axis, len(amps))
        tables[f"cie{axis}"] = from_spd(F(360), F(830), amps)
    ysum = F(0)
    for v in tables["cieY"]:
        ysum = ysum + v
    # the CIE daylight basis S0, S1, S2 as XYZ (s0XYZ/s1XYZ/s2XYZ,
    # Spectrum.hs:234-241), for chromaticityToXYZ (Spectrum.hs:243-251)
    cie = {axis: parse_list(src, f"cie{axis}Values") for axis in "XYZ"}
    s012 = []
    for name in ("cieS0", "cieS1", "cieS2"):
        s012 += spd_to_xyz(parse_spd(src, name), cie)

    lines = [
        "/* Generated by bling_gb300/gen_spectrum_tables.py from bling's Spectrum.hs.",
        " * 16-band values as GHC computes them at start-up (fromSpd/avgSpd,",
        " * Spectrum.hs:297-335); bit patterns are exact binary32. Do not edit. */",
        "#pragma once",
        "#include <stdint.h>",
        "#include <string.h>",
        "#ifndef BLING_HD",
        "#if defined(__CUDACC__)",
        "#define BLING_HD __host__ __device__",
        "#else",
        "#define BLING_HD",
        "#endif",
        "#endif",
        "static inline BLING_HD float __bling_f32(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }",
        "#define BLING_SPECTRUM_BANDS 16",
        "/* index order of the RGB basis tables below */",
        "enum { BLING_BASIS_WHITE, BLING_BASIS_CYAN, BLING_BASIS_MAGENTA, BLING_BASIS_YELLOW,",
        "       BLING_BASIS_RED, BLING_BASIS_GREEN, BLING_BASIS_BLUE };",
        "",
        "/* bit patterns, so the tables can live in __constant__ or host memory alike */",
    ]

    def emit(cname, vals):
        bits = [struct.unpack("<I", struct.pack("<f", float(v)))[0] for v in vals]
        lines.append(f"static const uint32_t {cname}[{len(bits)}] = {{")
        for k in range(0, len(bits), 4):
            chunk = ", ".join(f"0x{b:08x}u" for b in bits[k:k + 4])
            lines.append(f"   {chunk},")
        lines.append("};")

    emit("BLING_CIE_X_BITS", tables["cieX"])
    emit("BLING_CIE_Y_BITS", tables["cieY"])
    emit("BLING_CIE_Z_BITS", tables["cieZ"])
    lines.append(f"#define BLING_CIE_Y_SUM_BITS 0x{struct.unpack('<I', struct.pack('<f', float(ysum)))[0]:08x}u"
                 f" /* {float(ysum)!r} */")
    refl = [tables[n] for n in BASIS_NAMES[:7]]
    illum = [tables[n] for n in BASIS_NAMES[7:]]
    emit("BLING_RGB_REFL_BITS", [v for t in refl for v in t])
    emit("BLING_RGB_ILLUM_BITS", [v for t in illum for v in t])
    lines.append("/* X, Y, Z of the CIE daylight components S0, S1, S2 (spdToXYZ) */")
    emit("BLING_CIE_S012_XYZ_BITS", s012)
    # Perlin's permutation of noisePerms (Texture.hs:395-413), the list l of
    # `V.fromList (l ++ l)`; its second copy is index & 255
    tex = src_path.with_name("Texture.hs").read_text()
    m = re.search(r"^noisePerms\s*=.*?where\s*l\s*=\s*\[(.*?)\]", tex, re.S | re.M)
    if not m:
        raise SystemExit("noisePerms not found in Texture.hs")
    perm = [int(t) for t in m.group(1).replace("\n", " ").split(",") if t.strip()]
    assert sorted(perm) == list(range(256)), "noisePerms is not a permutation of 0..255"
    lines.append("/* noisePerms' permutation of 0..255 (Texture.hs:395-413), as an")
    lines.append(" * initializer list for host and device arrays */")
    lines.append("#define BLING_NOISE_PERM_LIST \\")
    for k in range(0, 256, 16):
        tail = ", \\" if k + 16 < 256 else ""
        lines.append("   " + ", ".join(str(v) for v in perm[k:k + 16]) + tail)
    lines.append("")
    out_path.write_text("\n".join(lines) + "\n")
    print(f"wrote {out_path}")


if __name__ == "__main__":
    main(sys.argv)
