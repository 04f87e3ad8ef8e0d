"""Affine/projective transforms for scene description, in IEEE binary32.

Restates bling's Transform.hs (and the camera set-up of Camera.hs) with one
rounding per operation in the reference's order, so the matrices handed to
the GPU are the ones a GHC build of the reference would compute:

* a transform is the pair (m, m^-1) of row-major 4x4 matrices
  (``MkTransform``, Transform.hs:124-127);
* ``concat(a, b)`` is ``a <> b`` -- apply ``a`` first, then ``b``
  (``concatTrans``/``mul``, Transform.hs:102-105, 241-244);
* ``invert`` is the reference's Gauss-Jordan elimination with full pivoting
  (Transform.hs:44-87), used by ``look_at`` and ``perspective``.

Transcendentals call the C library's ``sinf``/``cosf``/``tanf`` as GHC's Float
primops do.
"""
from __future__ import annotations

import ctypes
import ctypes.util

import numpy as np

F = np.float32
_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
for _fn in ("sinf", "cosf", "tanf", "sqrtf"):
    getattr(_libm, _fn).restype = ctypes.c_float
    getattr(_libm, _fn).argtypes = [ctypes.c_float]

PI = F(np.pi)


def sinf(x):
    return F(_libm.sinf(F(x)))


def cosf(x):
    return F(_libm.cosf(F(x)))


def tanf(x):
    return F(_libm.tanf(F(x)))


def radians(x):
    """radians x = x / 180 * pi (Math.hs:62-66)"""
    return F(F(x) / F(180)) * PI


class Transform:
    """(m, inv) pair; both float32 arrays of shape (16,), row-major."""

    __slots__ = ("m", "inv")

    def __init__(self, m, inv):
        self.m = np.asarray(m, dtype=np.float32).reshape(16).copy()
        self.inv = np.asarray(inv, dtype=np.float32).reshape(16).copy()

    def inverse(self) -> "Transform":
        return Transform(self.inv, self.m)

    def __matmul__(self, other: "Transform") -> "Transform":
        """``self <> other``: apply self first, then other."""
        return concat(self, other)

    def pack(self) -> np.ndarray:
        return np.concatenate([self.m, self.inv])


def _mul(m1, m2):
    """mul m1 m2 (Transform.hs:102-105): out[i][j] = sum_k m1[k][j] * m2[i][k]"""
    out = np.zeros(16, dtype=np.float32)
    for n in range(16):
        i, j = divmod(n, 4)
        s = F(0)
        for k in range(4):
            s = s + m1[k * 4 + j] * m2[i * 4 + k]
        out[n] = s
    return out


def invert(m):
    """Gauss-Jordan inversion (Transform.hs:44-87), binary32."""
    a = np.asarray(m, dtype=np.float32).copy()

    def idx(r, c):
        return c * 4 + r

    ipiv = [0, 1, 2, 3]
    steps = []
    for _ in range(4):
        best = None
        irow = icol = -1
        for j in ipiv:
            for k in ipiv:
                v = abs(a[idx(j, k)])
                # maximumBy keeps the later element unless strictly smaller
                if best is None or best < v or best == v:
                    best, irow, icol = v, j, k
        ipiv = [x for x in ipiv if x != icol]
        if irow != icol:
            for k in range(4):
                a[idx(irow, k)], a[idx(icol, k)] = a[idx(icol, k)], a[idx(irow, k)]
        pivinv = F(1) / a[idx(icol, icol)]
        a[idx(icol, icol)] = F(1)
        for j in range(4):
            a[idx(icol, j)] = a[idx(icol, j)] * pivinv
        for j in range(4):
            if j == icol:
                continue
            save = a[idx(j, icol)]
            a[idx(j, icol)] = F(0)
            for k in range(4):
                x = a[idx(icol, k)]
                old = a[idx(j, k)]
                a[idx(j, k)] = old - x * save
        steps.append((irow, icol))
    for ir, ic in reversed(steps):
        if ir != ic:
            for k in range(4):
                a[idx(k, ir)], a[idx(k, ic)] = a[idx(k, ic)], a[idx(k, ir)]
    return a


def concat(a: Transform, b: Transform) -> Transform:
    """concatTrans (Transform.hs:241-244)."""
    return Transform(_mul(a.m, b.m), _mul(b.inv, a.inv))


def identity() -> Transform:
    e = np.eye(4, dtype=np.float32).reshape(16)
    return Transform(e, e)


def translate(dx, dy, dz) -> Transform:
    dx, dy, dz = F(dx), F(dy), F(dz)
    m = [1, 0, 0, dx, 0, 1, 0, dy, 0, 0, 1, dz, 0, 0, 0, 1]
    i = [1, 0, 0, -dx, 0, 1, 0, -dy, 0, 0, 1, -dz, 0, 0, 0, 1]
    return Transform(m, i)


def scale(sx, sy, sz) -> Transform:
    sx, sy, sz = F(sx), F(sy), F(sz)
    m = [sx, 0, 0, 0, 0, sy, 0, 0, 0, 0, sz, 0, 0, 0, 0, 1]
    i = [F(1) / sx, 0, 0, 0, 0, F(1) / sy, 0, 0, 0, 0, F(1) / sz, 0, 0, 0, 0, 1]
    return Transform(m, i)


def _rot(axis: int, deg) -> Transform:
    s, c = sinf(radians(deg)), cosf(radians(deg))
    if axis == 0:
        m = [1, 0, 0, 0, 0, c, -s, 0, 0, s, c, 0, 0, 0, 0, 1]
    elif axis == 1:
        m = [c, 0, s, 0, 0, 1, 0, 0, -s, 0, c, 0, 0, 0, 0, 1]
    else:
        m = [c, -s, 0, 0, s, c, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1]
    m = np.asarray(m, dtype=np.float32)
    return Transform(m, m.reshape(4, 4).T.reshape(16))  # transMatrix m


def rotate_x(deg):
    return _rot(0, deg)


def rotate_y(deg):
    return _rot(1, deg)


def rotate_z(deg):
    return _rot(2, deg)


def _sqlen(v):
    return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]


def normalize(v):
    """normalize (Math.hs:349-353)"""
    v = [F(x) for x in v]
    if _sqlen(v) != 0:
        il = F(1) / F(_libm.sqrtf(_sqlen(v)))
        return [v[0] * il, v[1] * il, v[2] * il]
    return [F(0), F(1), F(0)]


def cross(u, v):
    return [u[1] * v[2] - u[2] * v[1], -(u[0] * v[2] - u[2] * v[0]), u[0] * v[1] - u[1] * v[0]]


def look_at(pos, look, up) -> Transform:
    """lookAt (Transform.hs:222-235)"""
    p = [F(x) for x in pos]
    l = [F(x) for x in look]
    u = [F(x) for x in up]
    d = normalize([l[0] - p[0], l[1] - p[1], l[2] - p[2]])
    left = normalize(cross(normalize(u), d))
    uu = cross(d, left)
    m = np.asarray([left[0], uu[0], d[0], p[0], left[1], uu[1], d[1], p[1],
                    left[2], uu[2], d[2], p[2], 0, 0, 0, 1], dtype=np.float32)
    return Transform(m, invert(m))


def perspective(fov, n, f) -> Transform:
    """perspective (Transform.hs:207-219)"""
    n, f = F(n), F(f)
    i_tan = F(1) / tanf(radians(fov) / F(2))
    m = np.asarray([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, f / (f - n), -(f * n) / (f - n), 0, 0, 1, 0],
                   dtype=np.float32)
    return concat(scale(i_tan, i_tan, 1), Transform(m, invert(m)))


def perspective_camera(c2w: Transform, lens_radius, focal_distance, fov, sx, sy, full=False):
    """mkPerspectiveCamera / mkProjective (Camera.hs:108-147): returns the
    (c2w, r2c) transforms the camera uses to fire rays; with full=True also
    the world-to-raster transform and the pixel area that sampleCam uses
    (w2r = (inverse c2w <> p) <> s2r, ap = pw * ph)."""
    p = perspective(fov, F(1e-2), F(1000))
    sx, sy = F(sx), F(sy)
    aspect = sx / sy
    if aspect > 1:
        s0, s1, s2, s3 = -aspect, aspect, F(-1), F(1)
    else:
        s0, s1, s2, s3 = F(-1), F(1), F(-1) / aspect, F(1) / aspect
    st1 = scale(sx, sy, 1)
    st2 = scale(F(1) / (s1 - s0), F(1) / (s2 - s3), 1)
    t = translate(-s0, -s3, 0)
    s2r = concat(t, concat(st2, st1))  # t <> st2 <> st1, (<>) is infixr
    r2c = concat(s2r.inverse(), p.inverse())
    if not full:
        return c2w, r2c
    w2r = concat(concat(c2w.inverse(), p), s2r)
    fl = tanf(radians(fov) / F(2))
    pw = fl * (s1 - s0) / sx
    ph = fl * (s3 - s2) / sy
    return c2w, r2c, w2r, F(pw * ph)
