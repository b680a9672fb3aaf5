"""3-D stencils over device grids (the role of ncarray's Stencil<3>,
src/lib/ncarray/expression/stencil.hh:58-255, for linear 3x3x3 stencils).

``Stencil3D(weights, dt).apply(src, dst)`` computes
    dst[z,y,x] = src[z,y,x] + dt * sum_{dz,dy,dx in -1..1} w[dz,dy,dx] * src[z+dz, y+dy, x+dx]
with zero halo; ``iterate(a, b, n)`` runs n Jacobi steps ping-ponging a <-> b
and returns the array holding the result.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .array import NCDevArray, current_stream


def laplacian7() -> np.ndarray:
    """6-neighbour Laplacian: -6 at the centre, +1 on the faces."""
    w = np.zeros((3, 3, 3))
    w[1, 1, 1] = -6.0
    for dz, dy, dx in ((0, 1, 1), (2, 1, 1), (1, 0, 1), (1, 2, 1), (1, 1, 0), (1, 1, 2)):
        w[dz, dy, dx] = 1.0
    return w


def laplacian27() -> np.ndarray:
    """27-point Laplacian (1/30)[-128 centre, 14 faces, 3 edges, 1 corners]."""
    w = np.zeros((3, 3, 3))
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                far = (dz != 1) + (dy != 1) + (dx != 1)
                w[dz, dy, dx] = {0: -128.0, 1: 14.0, 2: 3.0, 3: 1.0}[far] / 30.0
    return w


class Stencil3D:
    def __init__(self, weights, dt: float = 1.0):
        w = np.asarray(weights, dtype=np.float64).reshape(27)
        self._w = (ctypes.c_double * 27)(*w.tolist())
        self.dt = float(dt)

    def apply(self, src: NCDevArray, dst: NCDevArray) -> NCDevArray:
        _lib.call("nca_stencil3d", ctypes.byref(src.view_struct()), ctypes.byref(dst.view_struct()), self._w,
                  self.dt, current_stream())
        return dst

    def iterate(self, a: NCDevArray, b: NCDevArray, iters: int) -> NCDevArray:
        _lib.call("nca_stencil3d_iterate", ctypes.byref(a.view_struct()), ctypes.byref(b.view_struct()), self._w,
                  self.dt, int(iters), current_stream())
        return a if iters % 2 == 0 else b


def device_status() -> int:
    """Reads and clears the device status word of bounded waits (0 = ok)."""
    st = ctypes.c_int32(0)
    _lib.call("nca_device_status", ctypes.byref(st), current_stream())
    return st.value
