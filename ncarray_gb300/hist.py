"""2-D histogram binning of device point arrays (nca_hist2d).

``hist2d(x, y, nbx, nby, (x_lo, x_hi), (y_lo, y_hi), w=None)`` returns
``(counts uint64 (nby, nbx), wsum float32 (nby, nbx) or None)`` as new device
arrays; ``hist2d_into`` accumulates into existing ones.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Tuple

from . import _lib
from .array import NCDevArray, current_stream
from .dtype import DType


def _ptr(a: Optional[NCDevArray]):
    if a is None:
        return None
    if a.dtype != DType.float32 or not a.is_contiguous():
        raise TypeError("points and weights must be contiguous float32 arrays")
    return a.ptr


def hist2d_into(x: NCDevArray, y: NCDevArray, counts: NCDevArray, xr: Tuple[float, float],
                yr: Tuple[float, float], w: Optional[NCDevArray] = None, wsum: Optional[NCDevArray] = None) -> None:
    nby, nbx = counts.shape
    if x.size != y.size or (w is not None and w.size != x.size):
        raise ValueError("x, y (and w) must have the same length")
    if counts.dtype != DType.uint64 or not counts.is_contiguous():
        raise TypeError("counts must be a contiguous uint64 array")
    if wsum is not None and (wsum.dtype != DType.float32 or wsum.shape != counts.shape):
        raise TypeError("wsum must be float32 with the shape of counts")
    _lib.call("nca_hist2d", _ptr(x), _ptr(y), _ptr(w), x.size, nbx, nby, float(xr[0]), float(xr[1]), float(yr[0]),
              float(yr[1]), counts.ptr, wsum.ptr if wsum is not None else None, current_stream())


def hist2d(x: NCDevArray, y: NCDevArray, nbx: int, nby: int, xr=(0.0, 1.0), yr=(0.0, 1.0),
           w: Optional[NCDevArray] = None):
    counts = NCDevArray((nby, nbx), DType.uint64).fill(0)
    wsum = NCDevArray((nby, nbx), DType.float32).fill(0.0) if w is not None else None
    hist2d_into(x, y, counts, xr, yr, w, wsum)
    return counts, wsum
