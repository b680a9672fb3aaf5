"""Batched reductions over many 1-D device arrays of uneven length.

``Batch(arrays)`` prepares the descriptor table once; ``run()`` returns a
(n, 4) float64 device array of (sum, mean, max, sum(x*x - x)) per array from
one persistent launch (``graph=True`` replays it through a CUDA graph);
``run_plain()`` is the per-array, per-op float64 form; ``autotune()`` picks
and caches the schedule for this shape class.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

from . import _lib
from .array import NCDevArray, current_stream
from .dtype import DType


class Batch:
    def __init__(self, arrays: Sequence[NCDevArray]):
        self.arrays = list(arrays)   # keeps the device buffers alive
        items = (_lib.BatchItem * max(len(self.arrays), 1))()
        for i, a in enumerate(self.arrays):
            if a.dtype not in (DType.float32, DType.bfloat16, DType.float16) or not a.is_contiguous():
                raise TypeError("batched reductions take contiguous float32/bfloat16/float16 arrays")
            items[i].data = a.ptr
            items[i].length = a.size
            items[i].dtype = int(a.dtype)
        self._h = ctypes.c_void_p()
        _lib.call("nca_batch_create", items, len(self.arrays), ctypes.byref(self._h), current_stream())
        self.results = NCDevArray((len(self.arrays), 4), DType.float64)

    def run(self, graph: bool = False) -> NCDevArray:
        fn = "nca_batch_reduce_graph" if graph else "nca_batch_reduce"
        _lib.call(fn, self._h, self.results.ptr, current_stream())
        return self.results

    def run_plain(self) -> NCDevArray:
        _lib.call("nca_batch_reduce_plain", self._h, self.results.ptr, current_stream())
        return self.results

    def autotune(self) -> dict:
        _lib.call("nca_batch_autotune", self._h, self.results.ptr, current_stream())
        return self.schedule()

    def schedule(self) -> dict:
        c, t, u, n = ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _lib.call("nca_batch_schedule", self._h, ctypes.byref(c), ctypes.byref(t), ctypes.byref(u), ctypes.byref(n))
        return {"chunk_bytes": c.value, "threads": t.value, "items_per_thread": u.value, "ctas": n.value}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().nca_batch_destroy(h)
            except Exception:
                pass
            self._h = ctypes.c_void_p()
