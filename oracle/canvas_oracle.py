"""CPU restatement of the reference's 2D voxel canvas (test infrastructure only).

Only tests and the canvas benchmark's CPU leg use this file.  It restates
Canvas2D_CC (Canvas2D_CC.cpp:5-262) in float64 numpy, vectorised over the
voxels, with the reference's arithmetic order so that voxel membership is bit
for bit the reference's:

* the canvas has floor(size / offset) voxels per axis, voxel (ix, iy) at
  (ix, iy) * offset + 0.5 * offset (:5-30), numbered ix + iy * nx;
* circle / cutCircle test |p - c| = sqrt(dx dx + dy dy) against r (:43-56, :136-150);
* ring (:58-83) activates voxels with r_in + offset/2 <= d <= r_out - offset/2,
  marking those within one offset of either radius as surface unless the voxel
  was already active and not surface;
* rectangle / cutRectangle / prism (:85-134, :152-176) move the voxel into the
  shape's frame with the 4x4 transform rotate(-angle, z) * translate(-c)
  (glm's translate/rotate; the product's terms summed left to right) and test
  the local coordinates against the half sizes (the prism's y half size
  shrinks linearly with x by `extra`).

``apply(nx, ny, offset, ops)`` returns the voxel flags (bit 0 active, bit 1
surface); ops are tuples like ``("ring", cx, cy, r_out, r_in)``.
"""
from __future__ import annotations

import math
from typing import Iterable, Sequence, Tuple

import numpy as np

ACTIVE, SURFACE = 1, 2


def size(width: float, height: float, offset: float) -> Tuple[int, int]:
    return int(math.floor(width / offset)), int(math.floor(height / offset))


def positions(nx: int, ny: int, offset: float) -> np.ndarray:
    ix = np.tile(np.arange(nx, dtype=np.float64), ny)
    iy = np.repeat(np.arange(ny, dtype=np.float64), nx)
    return np.stack([ix * offset + 0.5 * offset, iy * offset + 0.5 * offset], axis=1)


def transform(cx: float, cy: float, angle: float) -> np.ndarray:
    """The 4x4 column-major matrix rotate(-angle, z) * translate(-c) of the rectangle ops (M[col][row])."""
    a = -angle
    cs, sn = math.cos(a), math.sin(a)
    n = (0.0, 0.0, 1.0)
    k = ((0.0, -n[2], n[1]), (n[2], 0.0, -n[0]), (-n[1], n[0], 0.0))
    R = [[1.0 if c == r else 0.0 for r in range(4)] for c in range(4)]
    for c in range(3):
        for r in range(3):
            R[c][r] = ((cs if c == r else 0.0) + (1.0 - cs) * n[r] * n[c]) + sn * k[r][c]
    T = [[1.0 if c == r else 0.0 for r in range(4)] for c in range(4)]
    T[3][0], T[3][1], T[3][2] = -cx, -cy, 0.0
    ident = [[1.0 if c == r else 0.0 for r in range(4)] for c in range(4)]

    def mul(A, B):
        return [[((A[0][r] * B[c][0] + A[1][r] * B[c][1]) + A[2][r] * B[c][2]) + A[3][r] * B[c][3]
                 for r in range(4)] for c in range(4)]

    return np.array(mul(mul(ident, R), T))


def local(p: np.ndarray, M: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """M * (x, y, 0, 1), rows 0 and 1, terms summed left to right."""
    x, y = p[:, 0], p[:, 1]
    lx = ((M[0][0] * x + M[1][0] * y) + M[2][0] * 0.0) + M[3][0] * 1.0
    ly = ((M[0][1] * x + M[1][1] * y) + M[2][1] * 0.0) + M[3][1] * 1.0
    return lx, ly


def apply(nx: int, ny: int, offset: float, ops: Iterable[Sequence], flags: np.ndarray = None) -> np.ndarray:
    p = positions(nx, ny, offset)
    f = np.zeros(nx * ny, dtype=np.uint8) if flags is None else flags.copy()
    for op in ops:
        kind, a = op[0], [float(v) for v in op[1:]]
        if kind in ("circle", "cutcircle", "ring"):
            dx, dy = p[:, 0] - a[0], p[:, 1] - a[1]
            d = np.sqrt(dx * dx + dy * dy)
            if kind == "circle":
                f[~(d > a[2])] |= ACTIVE
            elif kind == "cutcircle":
                f[~(d > a[2])] &= np.uint8(~ACTIVE & 0xFF)
            else:
                ro, ri = a[2], a[3]
                take = ~((d < ri + 0.5 * offset) | (ro - 0.5 * offset < d))
                surf = (np.abs(d - ro) < offset) | (np.abs(d - ri) < offset)
                was_active = (f & ACTIVE) != 0
                was_surface = (f & SURFACE) != 0
                surf = np.where(surf & was_active & ~was_surface, False, surf)
                nf = (f | ACTIVE) & np.uint8(~SURFACE & 0xFF)
                nf = np.where(surf, nf | SURFACE, nf)
                f = np.where(take, nf, f).astype(np.uint8)
        elif kind in ("rect", "cutrect", "prism"):
            sx, sy = a[2], a[3]
            rot = a[5] if kind == "prism" else a[4]
            lx, ly = local(p, transform(a[0], a[1], rot))
            out = (lx < -0.5 * sx) | (0.5 * sx < lx)
            if kind == "prism":
                extra = a[4]
                t = 0.5 * extra * (2.0 * lx / sx)
                out |= (ly < -0.5 * sy + t) | (0.5 * sy - t < ly)
            else:
                out |= (ly < -0.5 * sy) | (0.5 * sy < ly)
            if kind == "cutrect":
                f[~out] &= np.uint8(~ACTIVE & 0xFF)
            else:
                f[~out] |= ACTIVE
        else:
            raise ValueError(f"unknown canvas operation {kind!r}")
    return f
