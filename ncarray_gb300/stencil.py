"""Stencils over device arrays: ncarray's Stencil<NDIM>
(src/lib/ncarray/expression/stencil.hh:58-255).

``Stencil.create(offsets, op_func, dtype)`` mirrors the reference's
``Stencil<NDIM>::create<SrcT>(offsets, is_pointer_axis, op_func)``: op_func
receives one placeholder view per offset and returns an expression over them;
``apply(src, dest)`` evaluates
    dest[c] = expr(src[c*step + o_0], src[c*step + o_1], ...),  step = src.shape // dest.shape
through nca_stencil (any offsets, any dims, pointer-axis sources).

``Stencil3D(weights, dt)`` is the linear 3x3x3 special case on a dedicated
TMA-tiled kernel:
    dst[z,y,x] = src[z,y,x] + dt * sum_{dz,dy,dx in -1..1} w[dz,dy,dx] * src[z+dz, y+dy, x+dx]
with zero halo; ``iterate(a, b, n)`` runs n Jacobi steps ping-ponging a <-> b
and returns the array holding the result.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .array import DevExpr, NCDevArray, current_stream, lazy_mode
from .dtype import DType, FLOATS, arith, compute_dtype


class _Slot(NCDevArray):
    """Placeholder view handed to a stencil's op_func (no device memory): the
    expression records which offset each operand stands for."""

    def __init__(self, slot: int, dtype: DType, ndim: int):   # noqa: D401 - no buffer
        self.dtype = DType(dtype)
        self.shape = (1,) * ndim
        self.strides = (0,) * ndim
        self._offset = 0
        self._ptr = None
        self._slot = slot

    @property
    def ptr(self) -> int:
        return 1 + self._slot    # a distinct key per slot, never dereferenced


class Stencil:
    """A stencil of shifted views compiled once and applied to many arrays."""

    def __init__(self, offsets, instrs, scalars, compute, result, is_pointer_axis=None):
        self.ndim = len(offsets[0])
        self._offs = (ctypes.c_int64 * (len(offsets) * self.ndim))(*[int(v) for o in offsets for v in o])
        self.n = len(offsets)
        self.result_dtype = result
        self.is_pointer_axis = None if is_pointer_axis is None else [bool(x) for x in is_pointer_axis]
        self._ins = (ctypes.c_uint32 * len(instrs))(*instrs)
        self._sd = (ctypes.c_int32 * max(len(scalars), 1))(*[int(d) for d, _ in scalars])
        self._ss = (ctypes.c_uint64 * max(len(scalars), 1))(*[v for _, v in scalars])
        t = _lib.Tape()
        t.instrs = ctypes.cast(self._ins, ctypes.POINTER(ctypes.c_uint32))
        t.n_instrs = len(instrs)
        t.n_scalars = len(scalars)
        t.scalar_dtypes = ctypes.cast(self._sd, ctypes.POINTER(ctypes.c_int32))
        t.scalar_slots = ctypes.cast(self._ss, ctypes.POINTER(ctypes.c_uint64))
        t.compute_dtype = int(compute)
        t.result_dtype = int(result)
        self._tape = t

    @classmethod
    def create(cls, offsets, op_func, dtype: DType, is_pointer_axis=None) -> "Stencil":
        """offsets: a sequence of ndim-tuples; op_func(views) -> expression.
        Operand k of the returned expression reads offset k's view. Float
        expressions are evaluated in their work dtype, as the reference's
        generated stencil kernel does (rtcompiler.hh:187-385); integer ones in
        the expression's compute dtype."""
        offsets = [tuple(int(v) for v in o) for o in offsets]
        if not offsets or len({len(o) for o in offsets}) != 1:
            raise ValueError("offsets must be a non-empty list of equal-length tuples")
        ndim = len(offsets[0])
        slots = [_Slot(i, dtype, ndim) for i in range(len(offsets))]
        with lazy_mode():
            e = op_func(slots)
        if not isinstance(e, DevExpr):
            e = DevExpr.leaf(e) if isinstance(e, NCDevArray) else DevExpr.const(e)
        # operand k of the tape is the k-th distinct slot the expression loads
        used = [offsets[a._slot] for a in e.arrays]
        if not used:
            raise ValueError("the stencil expression reads no view")
        work = arith(e.work)
        compute = work if work in FLOATS else compute_dtype(e.expr_dtype, e.work)
        return cls(used, list(e.instrs), list(e.scalars), compute, e.expr_dtype, is_pointer_axis)

    def apply(self, src: NCDevArray, dest: NCDevArray, stream=None) -> NCDevArray:
        """dest[c] = expr(src[c * step + o] for each offset o). Does not
        synchronise (the reference's apply with a stream does not either)."""
        if src.ndim != self.ndim or dest.ndim != self.ndim:
            raise ValueError(f"stencil of {self.ndim} dims applied to {src.ndim}-d / {dest.ndim}-d arrays")
        if self.is_pointer_axis is not None:
            have = [src._ptr is not None and d == 0 for d in range(src.ndim)]
            if have != self.is_pointer_axis:
                raise ValueError("the source's pointer axes differ from those the stencil was created for")
        _lib.call("nca_stencil", ctypes.byref(src.view_struct()), ctypes.byref(dest.view_struct()), self._offs,
                  self.n, ctypes.byref(self._tape), current_stream() if stream is None else stream)
        return dest


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
