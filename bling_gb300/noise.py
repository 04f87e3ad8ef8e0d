"""Host-side noise for scene construction: Perlin noise and fBm in binary32
(Texture.hs:328-413), vectorised over numpy float32 arrays, for the scalar
maps that build geometry on the host (the `heightMap` primitive's
elevation, Heightmap.hs).  The textures a renderer evaluates per hit run on
the device (csrc/texture.cuh); this module only shapes meshes.

Every operation keeps the reference's order in float32 (numpy rounds each
float32 operation once and fuses nothing), and the permutation is the one
the table generator copied out of Texture.hs into spectrum_tables.h.
"""
from __future__ import annotations

import re
from pathlib import Path

import numpy as np

F = np.float32


def _perm() -> np.ndarray:
    text = (Path(__file__).with_name("csrc") / "spectrum_tables.h").read_text()
    m = re.search(r"#define BLING_NOISE_PERM_LIST((?:.*\\\n)*.*)", text)
    vals = [int(v) for v in re.findall(r"\d+", m.group(1))]
    assert sorted(vals) == list(range(256))
    return np.asarray(vals + vals, np.int64)  # noisePerms: the list twice


_P = _perm()


def _grad(x, y, z, dx, dy, dz):
    """grad (Texture.hs:384-393)"""
    h = _P[_P[_P[x] + y] + z] & 15
    u = np.where((h < 8) | (h == 12) | (h == 13), dx, dy)
    v = np.where((h < 4) | (h == 12) | (h == 13), dy, dz)
    return np.where(h & 1, -u, u) + np.where(h & 2, -v, v)


def _weight(t):
    """noiseWeight (Texture.hs:378-382)"""
    t3 = t * t * t
    t4 = t3 * t
    return F(6) * t4 * t - F(15) * t4 + F(10) * t3


def _lerp(t, a, b):
    return (F(1) - t) * a + t * b


def perlin3d(x, y, z) -> np.ndarray:
    """perlin3d (Texture.hs:348-376) of float32 arrays"""
    x, y, z = (np.asarray(v, F) for v in (x, y, z))
    fx, fy, fz = np.floor(x), np.floor(y), np.floor(z)
    dx, dy, dz = x - fx, y - fy, z - fz
    ix, iy, iz = (v.astype(np.int64) & 255 for v in (fx, fy, fz))
    one = F(1)
    w000 = _grad(ix, iy, iz, dx, dy, dz)
    w100 = _grad(ix + 1, iy, iz, dx - one, dy, dz)
    w010 = _grad(ix, iy + 1, iz, dx, dy - one, dz)
    w110 = _grad(ix + 1, iy + 1, iz, dx - one, dy - one, dz)
    w001 = _grad(ix, iy, iz + 1, dx, dy, dz - one)
    w101 = _grad(ix + 1, iy, iz + 1, dx - one, dy, dz - one)
    w011 = _grad(ix, iy + 1, iz + 1, dx, dy - one, dz - one)
    w111 = _grad(ix + 1, iy + 1, iz + 1, dx - one, dy - one, dz - one)
    wx, wy, wz = _weight(dx), _weight(dy), _weight(dz)
    y0 = _lerp(wy, _lerp(wx, w000, w100), _lerp(wx, w010, w110))
    y1 = _lerp(wy, _lerp(wx, w001, w101), _lerp(wx, w011, w111))
    return _lerp(wz, y0, y1)


def fbm(octaves: int, omega, x, y, z) -> np.ndarray:
    """fbm octaves omega (Texture.hs:328-337): the terms o_k * perlin3d(p
    l_k) summed from 0, l_k = 1.99^k and o_k = omega^k by repeated products"""
    x, y, z = (np.asarray(v, F) for v in (x, y, z))
    acc = np.zeros(np.broadcast(x, y, z).shape, F)
    l, o, omega = F(1), F(1), F(omega)
    for _ in range(octaves):
        acc = acc + o * perlin3d(x * l, y * l, z * l)
        l = F(1.99) * l
        o = omega * o
    return acc
