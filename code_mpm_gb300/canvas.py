"""Python front end of the GPU voxel canvas (include/mpm_canvas.h).

``Canvas2D`` mirrors the reference's ``Canvas2D_CC`` (Canvas2D_CC.h:28-76):
the same operation names and arguments, drawn on the GPU.  Drawing calls are
queued and applied in one pass at the next read; ``getVoxels_Active`` returns
the active voxels in voxel order as arrays (centres, ids, surface flags), to
host numpy arrays or, with ``device=True``, to torch CUDA tensors.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Tuple

import numpy as np

from . import engine

_SIGS = {
    "mpm_canvas_create": ([C.c_double, C.c_double, C.c_double, C.POINTER(C.c_void_p)], C.c_int),
    "mpm_canvas_destroy": ([C.c_void_p], C.c_int),
    "mpm_canvas_size": ([C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)], C.c_int),
    "mpm_canvas_last_error": ([C.c_void_p], C.c_char_p),
    "mpm_canvas_draw_circle": ([C.c_void_p] + [C.c_double] * 3, C.c_int),
    "mpm_canvas_draw_ring": ([C.c_void_p] + [C.c_double] * 4, C.c_int),
    "mpm_canvas_draw_rectangle": ([C.c_void_p] + [C.c_double] * 5, C.c_int),
    "mpm_canvas_draw_prism": ([C.c_void_p] + [C.c_double] * 6, C.c_int),
    "mpm_canvas_cut_circle": ([C.c_void_p] + [C.c_double] * 3, C.c_int),
    "mpm_canvas_cut_rectangle": ([C.c_void_p] + [C.c_double] * 5, C.c_int),
    "mpm_canvas_flags": ([C.c_void_p, C.c_void_p], C.c_int),
    "mpm_canvas_count_active": ([C.c_void_p, C.POINTER(C.c_uint64)], C.c_int),
    "mpm_canvas_active_voxels": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64,
                                  C.POINTER(C.c_uint64)], C.c_int),
}


def _lib():
    L = engine.lib()
    if not getattr(L, "_canvas_sigs", False):
        for name, (args, res) in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        L._canvas_sigs = True
    return L


class Canvas2D:
    """Canvas2D_CC(d2Size, dOffset) on the GPU."""

    def __init__(self, size: Tuple[float, float], offset: float):
        self._L = _lib()
        self._h = C.c_void_p()
        rc = self._L.mpm_canvas_create(float(size[0]), float(size[1]), float(offset), C.byref(self._h))
        if rc != 0:
            raise engine.MPMError(rc, "canvas creation failed")
        nx, ny = C.c_uint32(), C.c_uint32()
        self._L.mpm_canvas_size(self._h, C.byref(nx), C.byref(ny))
        self.d_Offset = float(offset)
        self.u2_Size = (int(nx.value), int(ny.value))

    def close(self) -> None:
        if self._h:
            self._L.mpm_canvas_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self) -> "Canvas2D":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int) -> None:
        if rc != 0:
            msg = self._L.mpm_canvas_last_error(self._h)
            raise engine.MPMError(rc, msg.decode() if msg else "")

    # -- drawing (Canvas2D_CC.cpp:43-176) ----------------------------------------------
    def drawCircle(self, center, radius: float) -> None:
        self._check(self._L.mpm_canvas_draw_circle(self._h, float(center[0]), float(center[1]), float(radius)))

    def drawRing(self, center, radius_outer: float, radius_inner: float) -> None:
        self._check(self._L.mpm_canvas_draw_ring(self._h, float(center[0]), float(center[1]), float(radius_outer),
                                                 float(radius_inner)))

    def drawRectangle(self, center, size, rotation: float = 0.0) -> None:
        self._check(self._L.mpm_canvas_draw_rectangle(self._h, float(center[0]), float(center[1]), float(size[0]),
                                                      float(size[1]), float(rotation)))

    def drawPrism(self, center, size, extra: float, rotation: float = 0.0) -> None:
        self._check(self._L.mpm_canvas_draw_prism(self._h, float(center[0]), float(center[1]), float(size[0]),
                                                  float(size[1]), float(extra), float(rotation)))

    def cutCircle(self, center, radius: float) -> None:
        self._check(self._L.mpm_canvas_cut_circle(self._h, float(center[0]), float(center[1]), float(radius)))

    def cutRectangle(self, center, size, rotation: float = 0.0) -> None:
        self._check(self._L.mpm_canvas_cut_rectangle(self._h, float(center[0]), float(center[1]), float(size[0]),
                                                     float(size[1]), float(rotation)))

    def apply_ops(self, ops) -> None:
        """Queue operations given as tuples, e.g. ("ring", cx, cy, r_out, r_in) (names as in the canvas oracle)."""
        for op in ops:
            k, a = op[0], op[1:]
            if k == "circle":
                self.drawCircle(a[:2], a[2])
            elif k == "ring":
                self.drawRing(a[:2], a[2], a[3])
            elif k == "rect":
                self.drawRectangle(a[:2], a[2:4], a[4])
            elif k == "prism":
                self.drawPrism(a[:2], a[2:4], a[4], a[5])
            elif k == "cutcircle":
                self.cutCircle(a[:2], a[2])
            elif k == "cutrect":
                self.cutRectangle(a[:2], a[2:4], a[4])
            else:
                raise ValueError(f"unknown canvas operation {k!r}")

    # -- reads --------------------------------------------------------------------------
    def flags(self) -> np.ndarray:
        """Voxel flags in voxel order (bit 0 active, bit 1 surface)."""
        out = np.zeros(self.u2_Size[0] * self.u2_Size[1], dtype=np.uint8)
        self._check(self._L.mpm_canvas_flags(self._h, out.ctypes.data))
        return out

    def getCount_Active(self) -> int:
        n = C.c_uint64()
        self._check(self._L.mpm_canvas_count_active(self._h, C.byref(n)))
        return int(n.value)

    def getVoxels_Active(self, device: bool = False) -> Dict[str, object]:
        """Active voxels in voxel order: centres "xy" (n x 2), "ids", "surface" (0/1)."""
        n = self.getCount_Active()
        if device:
            import torch

            xy = torch.empty((n, 2), dtype=torch.float64, device="cuda")
            ids = torch.empty((n,), dtype=torch.int32, device="cuda")
            surf = torch.empty((n,), dtype=torch.uint8, device="cuda")
            ptrs = (xy.data_ptr(), ids.data_ptr(), surf.data_ptr()) if n else (None, None, None)
        else:
            xy = np.zeros((n, 2))
            ids = np.zeros(n, dtype=np.uint32)
            surf = np.zeros(n, dtype=np.uint8)
            ptrs = (xy.ctypes.data, ids.ctypes.data, surf.ctypes.data)
        got = C.c_uint64()
        self._check(self._L.mpm_canvas_active_voxels(self._h, *ptrs, n, C.byref(got)))
        return {"xy": xy, "ids": ids, "surface": surf}
