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


class BatchExpr:
    """General batched reductions: ``items`` is a list of ``(array, outputs)``
    with ``outputs`` a list of up to four ``(fn, RedOp)`` pairs, ``fn`` a
    function of one placeholder element-expression (``lambda x: x * x - x``) or
    None for the element itself. One persistent launch computes every output of
    every item; ``run()`` returns an (n_items, 4, 2) float64/int64 view pair
    ``(values, indices)`` as numpy arrays after copying them back.

    A tape is built once per (fn, input dtype) with this package's ncarray
    expression rules and must have a float32 or float64 result."""

    def __init__(self, items):
        from .array import DevExpr, lazy_mode
        from .dtype import compute_dtype
        from .stencil import _Slot
        self.arrays = [a for a, _ in items]
        tape_key: dict = {}
        self._tapes = []     # (instrs, scalars, compute, result)
        citems = (_lib.BatchExprItem * max(len(items), 1))()
        for i, (a, outs) in enumerate(items):
            if not a.is_contiguous() or a.ndim != 1:
                raise TypeError("batched items are contiguous 1-D arrays")
            if not 1 <= len(outs) <= _lib.BATCH_MAX_OUTS:
                raise ValueError(f"1..{_lib.BATCH_MAX_OUTS} outputs per item")
            citems[i].data = a.ptr if a.size else None
            citems[i].length = a.size
            citems[i].dtype = int(a.dtype)
            citems[i].n_outs = len(outs)
            for o, (fn, op) in enumerate(outs):
                key = (fn, int(a.dtype))
                if key not in tape_key:
                    slot = _Slot(0, a.dtype, 1)
                    with lazy_mode():
                        e = DevExpr.leaf(slot) if fn is None else fn(DevExpr.leaf(slot))
                    if not isinstance(e, DevExpr):
                        raise TypeError("an output function must return an expression of its argument")
                    res = e.expr_dtype
                    if res not in (DType.float32, DType.float64, DType.bfloat16, DType.float16):
                        raise TypeError(f"batched outputs need a floating result (got {res.name})")
                    if res in (DType.bfloat16, DType.float16):
                        res = DType.float32
                    tape_key[key] = len(self._tapes)
                    self._tapes.append((list(e.instrs), list(e.scalars), compute_dtype(res, e.work), res))
                citems[i].tape[o] = tape_key[key]
                citems[i].op[o] = int(op)
        self.n = len(items)
        self._keep = []
        tapes = (_lib.Tape * len(self._tapes))()
        for k, (ins, sc, cdt, rdt) in enumerate(self._tapes):
            ia = (ctypes.c_uint32 * len(ins))(*ins)
            sd = (ctypes.c_int32 * max(len(sc), 1))(*[int(d) for d, _ in sc])
            ss = (ctypes.c_uint64 * max(len(sc), 1))(*[v for _, v in sc])
            self._keep += [ia, sd, ss]
            tapes[k].instrs = ctypes.cast(ia, ctypes.POINTER(ctypes.c_uint32))
            tapes[k].n_instrs = len(ins)
            tapes[k].n_scalars = len(sc)
            tapes[k].scalar_dtypes = ctypes.cast(sd, ctypes.POINTER(ctypes.c_int32))
            tapes[k].scalar_slots = ctypes.cast(ss, ctypes.POINTER(ctypes.c_uint64))
            tapes[k].compute_dtype = int(cdt)
            tapes[k].result_dtype = int(rdt)
        self._h = ctypes.c_void_p()
        _lib.call("nca_batch_expr_create", citems, self.n, tapes, len(self._tapes), ctypes.byref(self._h),
                  current_stream())
        # rows of (float64 value, int64 index): 16 bytes each
        self.results = NCDevArray((max(self.n, 1) * _lib.BATCH_MAX_OUTS * 2,), DType.int64)

    def launch(self, graph: bool = True, plain: bool = False) -> None:
        fn = "nca_batch_expr_run_plain" if plain else ("nca_batch_expr_run_graph" if graph else "nca_batch_expr_run")
        _lib.call(fn, self._h, self.results.ptr, current_stream())

    def run(self, graph: bool = True, plain: bool = False):
        """(values (n, 4) float64, indices (n, 4) int64) on the host."""
        import numpy as np
        self.launch(graph=graph, plain=plain)
        raw = self.results.to_host().view(np.uint8)[: self.n * _lib.BATCH_MAX_OUTS * 16]
        rec = raw.view(np.dtype([("value", "<f8"), ("index", "<i8")])).reshape(self.n, _lib.BATCH_MAX_OUTS)
        return rec["value"].copy(), rec["index"].copy()

    def info(self) -> dict:
        c, p, n = ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()
        _lib.call("nca_batch_expr_info", self._h, ctypes.byref(c), ctypes.byref(p), ctypes.byref(n))
        return {"chunks": c.value, "programs": p.value, "ctas": n.value}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().nca_batch_expr_destroy(h)
            except Exception:
                pass
            self._h = ctypes.c_void_p()
