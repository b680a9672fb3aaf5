"""Device arrays and lazy expressions with ncarray's Python surface.

Mirrors the classes of ncarray's ``_pyncdevarray`` module
(src/lib/pyncarray/ncdevarray.cu:47-58, binding_builder.hh:163-815):
``NCDevArray`` (owner or view over device memory), ``DevExpr`` (the lazy tape
of ExprMVNode, expression/mvnode.hh:82-459), the operator set, reductions
``sum/mean/max/min/argmax/argmin`` with and without axes, ``fill``,
``to_host``/``to_device`` and ``__array__``. Every device operation goes
through the C ABI of libncgb300; device memory is a torch byte buffer.
"""
from __future__ import annotations

import contextlib
import ctypes
from typing import Iterable, Optional, Sequence

import numpy as np

from . import _lib
from .dtype import (DType, FLOATS, ITEMSIZE, OpCode, RedOp, arith, compute_dtype, promote,
                    result_dtype, scalar_dtype, scalar_slot, sum_type, to_numpy)

_EAGER = [True]


def set_eager(flag: bool) -> None:
    """Eager mode materialises every operator result (ncarray's default)."""
    _EAGER[0] = bool(flag)


@contextlib.contextmanager
def lazy_mode():
    """Operators return DevExpr tapes that fuse into one kernel on use."""
    old = _EAGER[0]
    _EAGER[0] = False
    try:
        yield
    finally:
        _EAGER[0] = old


def _torch():
    import torch
    return torch


def current_stream() -> int:
    torch = _torch()
    return int(torch.cuda.current_stream().cuda_stream)


def _device():
    torch = _torch()
    if not torch.cuda.is_available():
        raise RuntimeError("ncarray_gb300 device arrays need a CUDA device")
    return torch.device("cuda", torch.cuda.current_device())


def _c_strides(shape: Sequence[int], itemsize: int) -> list[int]:
    st, acc = [], itemsize
    for n in reversed(shape):
        st.append(acc)
        acc *= max(int(n), 1)
    return list(reversed(st))


class NCDevArray:
    """An N-d device array (owner, or a strided view sharing an owner's buffer)."""

    def __init__(self, shape: Sequence[int] = (), dtype: DType = DType.float64, *, _buf=None,
                 _offset: int = 0, _strides: Optional[Sequence[int]] = None):
        self.dtype = DType(dtype)
        self.shape = tuple(int(n) for n in shape)
        isz = ITEMSIZE[self.dtype]
        if _buf is None:
            nbytes = max(self.size * isz, 1)
            _buf = _torch().empty(nbytes, dtype=_torch().uint8, device=_device())
        self._buf = _buf
        self._offset = int(_offset)
        self.strides = tuple(int(s) for s in (_strides if _strides is not None else _c_strides(self.shape, isz)))
        # pointer-axis views (from_panels): axis 0 indexes a device table of
        # panel pointers; None for ordinary arrays
        self._ptr = None

    # ---- metadata ----
    @property
    def ndim(self) -> int:
        return len(self.shape)

    @property
    def size(self) -> int:
        n = 1
        for e in self.shape:
            n *= e
        return n

    @property
    def itemsize(self) -> int:
        return ITEMSIZE[self.dtype]

    @property
    def nbytes(self) -> int:
        return self.size * self.itemsize

    @property
    def ptr(self) -> int:
        return int(self._buf.data_ptr()) + self._offset

    def is_contiguous(self) -> bool:
        return self._ptr is None and list(self.strides) == _c_strides(self.shape, self.itemsize)

    def view_struct(self) -> _lib.View:
        v = _lib.make_view(self.ptr, self.dtype, self.shape, self.strides)
        if self._ptr is not None:
            v.pointer_axis = 0
            if self._ptr["step"] == 1:
                # NC: the view's data is the first table entry; later axes' offsets
                # land on the panel side
                if self.ndim > 1:
                    v.offsets[1] = self._ptr["poff"]
            else:
                # a stepped table: SO semantics (stride along the table, suboffset)
                v.flags = _lib.VIEW_SUBOFFSETS
                v.offsets[0] = self._ptr["poff"]
        return v

    @classmethod
    def from_panels(cls, panels: Sequence["NCDevArray"]) -> "NCDevArray":
        """An array of shape (len(panels), *panel.shape) whose axis 0 is a
        pointer axis: element [i, ...] lives in panels[i] (ncarray's NCArray with
        a pointer axis, src/lib/ncarray/layout.hh:451-535). The panels share
        shape, dtype and strides; they are kept alive by the result."""
        panels = list(panels)
        if not panels:
            raise ValueError("at least one panel")
        p0 = panels[0]
        for p in panels:
            if p._ptr is not None or p.shape != p0.shape or p.dtype != p0.dtype or p.strides != p0.strides:
                raise ValueError("panels must be ordinary arrays of one shape, dtype and strides")
        table = cls.from_host(np.array([p.ptr for p in panels], dtype=np.uint64))
        out = cls((len(panels),) + p0.shape, p0.dtype, _buf=table._buf, _offset=table._offset,
                  _strides=(8,) + p0.strides)
        out._ptr = {"table": table, "panels": panels, "poff": 0, "step": 1}
        return out

    def __len__(self) -> int:
        return self.shape[0]

    def __repr__(self) -> str:
        return f"NCDevArray(shape={self.shape}, dtype={self.dtype.name})"

    # ---- construction ----
    @classmethod
    def empty(cls, shape: Sequence[int], dtype: DType) -> "NCDevArray":
        return cls(shape, dtype)

    @classmethod
    def from_host(cls, arr: np.ndarray, dtype: Optional[DType] = None) -> "NCDevArray":
        """Copies a numpy array to a new C-contiguous device owner.
        bfloat16 data is passed as uint16 bit patterns with dtype=DType.bfloat16."""
        from .dtype import from_numpy
        a = np.ascontiguousarray(arr)
        dt = DType(dtype) if dtype is not None else from_numpy(a.dtype)
        if ITEMSIZE[dt] != a.itemsize:
            raise TypeError(f"{a.dtype} cannot hold {dt.name}")
        out = cls(a.shape, dt)
        if a.size:
            torch = _torch()
            src = torch.from_numpy(a.reshape(-1).view(np.uint8))
            out._buf[: a.nbytes].copy_(src, non_blocking=False)
        return out

    def to_host(self) -> np.ndarray:
        """Copies to a new C-contiguous numpy array (synchronises)."""
        src = self if self.is_contiguous() else self.copy()
        npdt = to_numpy(self.dtype)
        if src.size == 0:
            return np.zeros(self.shape, dtype=npdt)
        raw = src._buf[src._offset: src._offset + src.nbytes].cpu().numpy()
        return raw.view(npdt).reshape(self.shape)

    # ---- host <-> device copies of views (nca_copy_host) ----
    def _host_view(self, host) -> _lib.View:
        """A View of a host numpy array or CPU torch tensor with this array's
        shape and itemsize (pinned torch memory makes the copy asynchronous)."""
        if isinstance(host, np.ndarray):
            ptr, itemsize, strides = host.ctypes.data, host.itemsize, tuple(host.strides)
        else:
            if host.is_cuda:
                raise TypeError("host buffer expected")
            itemsize = host.element_size()
            ptr, strides = host.data_ptr(), tuple(st * itemsize for st in host.stride())
        if tuple(host.shape) != tuple(self.shape) or itemsize != self.itemsize:
            raise ValueError(f"host buffer {tuple(host.shape)} x {itemsize} B does not match {self.shape} x "
                             f"{self.itemsize} B")
        return _lib.make_view(ptr, self.dtype, self.shape, strides)

    def copy_from(self, host, stream=None) -> "NCDevArray":
        """self[...] = host (same shape and itemsize) on `stream` (default: the
        current stream); both views contiguous along their innermost axis."""
        hv = self._host_view(host)
        _lib.call("nca_copy_host", ctypes.byref(hv), ctypes.byref(self.view_struct()),
                  current_stream() if stream is None else stream)
        return self

    def copy_to(self, host, stream=None) -> None:
        """host[...] = self (same shape and itemsize) on `stream`; asynchronous
        with pinned host memory (synchronise before reading it)."""
        hv = self._host_view(host)
        _lib.call("nca_copy_host", ctypes.byref(self.view_struct()), ctypes.byref(hv),
                  current_stream() if stream is None else stream)

    def __array__(self, dtype=None, copy=None):
        a = self.to_host()
        return a.astype(dtype) if dtype is not None else a

    # ---- views ----
    def transpose(self, *axes) -> "NCDevArray":
        if self._ptr is not None:
            raise NotImplementedError("pointer-axis arrays keep their axis order; copy() them first")
        if len(axes) == 1 and isinstance(axes[0], (tuple, list)):
            axes = tuple(axes[0])
        if not axes:
            axes = tuple(reversed(range(self.ndim)))
        if sorted(axes) != list(range(self.ndim)):
            raise ValueError("axes must be a permutation")
        return NCDevArray([self.shape[a] for a in axes], self.dtype, _buf=self._buf,
                          _offset=self._offset, _strides=[self.strides[a] for a in axes])

    permute = transpose

    def reshape(self, *shape) -> "NCDevArray":
        if self._ptr is not None:
            raise NotImplementedError("pointer-axis arrays keep their axis order; copy() them first")
        if len(shape) == 1 and isinstance(shape[0], (tuple, list)):
            shape = tuple(shape[0])
        shape = list(shape)
        if -1 in shape:
            known = 1
            for s in shape:
                if s != -1:
                    known *= s
            shape[shape.index(-1)] = self.size // known
        n = 1
        for s in shape:
            n *= s
        if n != self.size:
            raise ValueError("reshape changes the size")
        src = self if self.is_contiguous() else self.copy()
        return NCDevArray(shape, self.dtype, _buf=src._buf, _offset=src._offset)

    def broadcast_to(self, shape: Sequence[int]) -> "NCDevArray":
        if self._ptr is not None:
            raise NotImplementedError("pointer-axis arrays keep their axis order; copy() them first")
        shape = tuple(shape)
        pad = len(shape) - self.ndim
        st = [0] * pad + list(self.strides)
        sh = [1] * pad + list(self.shape)
        for d in range(len(shape)):
            if sh[d] == 1 and shape[d] != 1:
                st[d] = 0
            elif sh[d] != shape[d]:
                raise ValueError("cannot broadcast")
        return NCDevArray(shape, self.dtype, _buf=self._buf, _offset=self._offset, _strides=st)

    def _ptr_getitem(self, key) -> "NCDevArray":
        """Indexing of a pointer-axis array: an integer on axis 0 selects a
        panel (an ordinary array); slices on axis 0 select table entries; the
        other axes slice every panel alike."""
        key = key + (slice(None),) * (self.ndim - len(key))
        if len(key) > self.ndim or any(k is None or k is Ellipsis for k in key):
            raise IndexError("pointer-axis arrays take one index or slice per axis")
        k0, rest = key[0], key[1:]
        if not isinstance(k0, slice):
            i = int(k0)
            if i < 0:
                i += self.shape[0]
            if not 0 <= i < self.shape[0]:
                raise IndexError("index out of range")
            panel = self._ptr["panels"][self._ptr.get("first", 0) + i * self._ptr["step"]]
            inner = NCDevArray(self.shape[1:], self.dtype, _buf=panel._buf,
                               _offset=panel._offset + self._ptr["poff"], _strides=self.strides[1:])
            return inner[rest] if rest else inner
        start, stop, step = k0.indices(self.shape[0])
        cnt = max(0, (stop - start + (step - (1 if step > 0 else -1))) // step)
        if step < 0:
            raise IndexError("negative steps on the pointer axis are not supported")
        # the inner axes as a probe view (offset 0) to get their shape/strides/offset
        probe = NCDevArray(self.shape[1:], self.dtype, _buf=self._buf, _offset=0, _strides=self.strides[1:])[rest] \
            if rest else NCDevArray(self.shape[1:], self.dtype, _buf=self._buf, _offset=0, _strides=self.strides[1:])
        out = NCDevArray((cnt,) + probe.shape, self.dtype, _buf=self._buf, _offset=self._offset + start * self.strides[0],
                         _strides=(self.strides[0] * step,) + probe.strides)
        out._ptr = dict(self._ptr)
        out._ptr["poff"] = self._ptr["poff"] + probe._offset
        out._ptr["step"] = self._ptr["step"] * step
        out._ptr["first"] = self._ptr.get("first", 0) + start * self._ptr["step"]
        return out

    def __getitem__(self, key) -> "NCDevArray":
        if not isinstance(key, tuple):
            key = (key,)
        if self._ptr is not None:
            return self._ptr_getitem(key)
        if Ellipsis in key:
            i = key.index(Ellipsis)
            key = key[:i] + (slice(None),) * (self.ndim - len(key) + 1) + key[i + 1:]
        shape, strides, off = [], [], self._offset
        d = 0
        for k in key:
            if k is None:
                shape.append(1)
                strides.append(0)
                continue
            n, s = self.shape[d], self.strides[d]
            if isinstance(k, slice):
                start, stop, step = k.indices(n)
                cnt = max(0, (stop - start + (step - (1 if step > 0 else -1))) // step)
                off += start * s
                shape.append(cnt)
                strides.append(s * step)
            else:
                i = int(k)
                if i < 0:
                    i += n
                if not 0 <= i < n:
                    raise IndexError("index out of range")
                off += i * s
            d += 1
        shape += list(self.shape[d:])
        strides += list(self.strides[d:])
        return NCDevArray(shape, self.dtype, _buf=self._buf, _offset=off, _strides=strides)

    def __setitem__(self, key, value) -> None:
        self[key].assign(value)

    # ---- copies ----
    def copy(self) -> "NCDevArray":
        out = NCDevArray(self.shape, self.dtype)
        out.assign(self)
        return out

    def astype(self, dtype: DType) -> "NCDevArray":
        out = NCDevArray(self.shape, dtype)
        out.assign(self)
        return out

    def assign(self, other) -> "NCDevArray":
        """Casting copy into this view (broadcasting `other`)."""
        if isinstance(other, DevExpr):
            other.evaluate(out=self)
            return self
        if isinstance(other, np.ndarray):
            other = NCDevArray.from_host(other)
        if isinstance(other, NCDevArray):
            if self.size:
                _lib.call("nca_copy", ctypes.byref(other.view_struct()), ctypes.byref(self.view_struct()),
                          current_stream())
            return self
        return self.fill(other)

    def fill(self, value) -> "NCDevArray":
        dt = scalar_dtype(value)
        slot = ctypes.c_uint64(scalar_slot(value, dt))
        if self.size:
            _lib.call("nca_fill", ctypes.byref(self.view_struct()), int(dt), ctypes.byref(slot), current_stream())
        return self

    def scatter_add(self, indices, src) -> "NCDevArray":
        """self[indices[i]] += src[i] for every element i (indices outside
        [0, len(self)) are dropped); self is 1-D, indices and src have one
        shape. Host (numpy) indices or sources are copied to the device first,
        as the reference binding does (pyncarray/binding_builder.hh:708-775)."""
        if isinstance(indices, np.ndarray):
            indices = NCDevArray.from_host(indices)
        if isinstance(src, np.ndarray):
            src = NCDevArray.from_host(src)
        _lib.call("nca_scatter_add", ctypes.byref(self.view_struct()), ctypes.byref(indices.view_struct()),
                  ctypes.byref(src.view_struct()), current_stream())
        return self

    # ---- expressions ----
    def _expr(self) -> "DevExpr":
        return DevExpr.leaf(self)

    # ---- reductions ----
    def sum(self, axes=None):
        return self._expr().sum(axes)

    def mean(self, axes=None):
        return self._expr().mean(axes)

    def max(self, axes=None):
        return self._expr().max(axes)

    def min(self, axes=None):
        return self._expr().min(axes)

    def argmax(self, axes=None):
        return self._expr().argmax(axes)

    def argmin(self, axes=None):
        return self._expr().argmin(axes)


def _as_node(x):
    if isinstance(x, DevExpr):
        return x
    if isinstance(x, NCDevArray):
        return DevExpr.leaf(x)
    if isinstance(x, np.ndarray):
        return DevExpr.leaf(NCDevArray.from_host(x))
    return DevExpr.const(x)


class DevExpr:
    """A lazy tape (RPN instructions over array operands and scalars)."""

    def __init__(self):
        self.arrays: list[NCDevArray] = []
        self.scalars: list[tuple[DType, int]] = []
        self.instrs: list[int] = []
        self.work: Optional[DType] = None
        self.expr_dtype: Optional[DType] = None

    # ---- building (ExprMVNode::build_node) ----
    @classmethod
    def leaf(cls, a: NCDevArray) -> "DevExpr":
        e = cls()
        e.arrays.append(a)
        e.instrs.append((OpCode.LOAD_NCARR << 24) | 0)
        e.work = e.expr_dtype = a.dtype
        return e

    @classmethod
    def const(cls, v) -> "DevExpr":
        e = cls()
        dt = scalar_dtype(v)
        e.scalars.append((dt, scalar_slot(v, dt)))
        e.instrs.append((OpCode.LOAD_CONST << 24) | 0)
        e.work = e.expr_dtype = dt
        return e

    @classmethod
    def iota(cls, like: "NCDevArray | Sequence[int]", dtype: DType = DType.int64) -> "DevExpr":
        """The IDX generator: the C-order linear index of each element."""
        shape = like.shape if isinstance(like, NCDevArray) else tuple(like)
        e = cls()
        e.instrs.append(OpCode.IDX << 24)
        e.work = e.expr_dtype = DType(dtype)
        e._iota_shape = tuple(shape)
        return e

    def _append(self, other: "DevExpr") -> None:
        # an operand view that is already on the tape is loaded through the same
        # index (one load per element instead of two)
        keys = {_view_key(a): i for i, a in enumerate(self.arrays)}
        remap = []
        for a in other.arrays:
            k = _view_key(a)
            if k not in keys:
                keys[k] = len(self.arrays)
                self.arrays.append(a)
            remap.append(keys[k])
        ns = len(self.scalars)
        self.scalars += other.scalars
        for ins in other.instrs:
            op, idx = ins >> 24, ins & 0xFFFFFF
            if op in (OpCode.LOAD_NCARR, OpCode.LOAD_SOARR):
                ins = (op << 24) | remap[idx]
            elif op == OpCode.LOAD_CONST:
                ins = (op << 24) | (idx + ns)
            self.instrs.append(ins)
        if getattr(other, "_iota_shape", None) is not None and getattr(self, "_iota_shape", None) is None:
            self._iota_shape = other._iota_shape

    def _clone(self) -> "DevExpr":
        e = DevExpr()
        e.arrays = list(self.arrays)
        e.scalars = list(self.scalars)
        e.instrs = list(self.instrs)
        e.work, e.expr_dtype = self.work, self.expr_dtype
        if getattr(self, "_iota_shape", None) is not None:
            e._iota_shape = self._iota_shape
        return e

    def _binary(self, op: OpCode, other, reverse: bool = False):
        a, b = (self, _as_node(other)) if not reverse else (_as_node(other), self)
        e = a._clone()
        e._append(b)
        e.work = promote(a.work, b.work)
        e.expr_dtype = result_dtype(op, e.work)
        e.instrs.append(op << 24)
        return e._finish()

    def _unary(self, op: OpCode):
        e = self._clone()
        e.expr_dtype = result_dtype(op, e.work)
        e.instrs.append(op << 24)
        return e._finish()

    def _finish(self):
        return self.materialize() if _EAGER[0] else self

    # ---- evaluation ----
    @property
    def dtype(self) -> DType:
        return self.expr_dtype

    @property
    def shape(self) -> tuple:
        shapes = [a.shape for a in self.arrays]
        if getattr(self, "_iota_shape", None) is not None:
            shapes.append(self._iota_shape)
        n = max((len(s) for s in shapes), default=0)
        out = [1] * n
        for s in shapes:
            for d, e in enumerate(s):
                ld = d + n - len(s)
                if e != 1:
                    if out[ld] not in (1, e):
                        raise ValueError("operands do not broadcast")
                    out[ld] = e
        return tuple(out)

    def _tape(self):
        ins = (ctypes.c_uint32 * max(len(self.instrs), 1))(*self.instrs)
        sd = (ctypes.c_int32 * max(len(self.scalars), 1))(*[int(d) for d, _ in self.scalars])
        ss = (ctypes.c_uint64 * max(len(self.scalars), 1))(*[s for _, s in self.scalars])
        t = _lib.Tape()
        t.instrs = ctypes.cast(ins, ctypes.POINTER(ctypes.c_uint32))
        t.n_instrs = len(self.instrs)
        t.n_scalars = len(self.scalars)
        t.scalar_dtypes = ctypes.cast(sd, ctypes.POINTER(ctypes.c_int32))
        t.scalar_slots = ctypes.cast(ss, ctypes.POINTER(ctypes.c_uint64))
        t.compute_dtype = int(compute_dtype(self.expr_dtype, self.work))
        t.result_dtype = int(self.expr_dtype)
        return t, (ins, sd, ss)

    def _operands(self):
        n = len(self.arrays)
        arr = (_lib.View * max(n, 1))(*[a.view_struct() for a in self.arrays])
        return arr, n

    def materialize(self) -> NCDevArray:
        out = NCDevArray(self.shape, self.expr_dtype)
        self.evaluate(out=out)
        return out

    def _abi(self):
        # the tape and operand descriptors never change once an expression is
        # built (operators return new objects), so they are packed once
        c = getattr(self, "_abi_cache", None)
        if c is None:
            t, keep = self._tape()
            ops, n = self._operands()
            c = self._abi_cache = (t, keep, ops, n)
        return c

    def evaluate(self, out: Optional[NCDevArray] = None, reductions: Iterable = (), red_out=None):
        """One fused pass: stores the value into `out` (if given) and computes
        the reductions, a sequence of (RedOp, axes or None). Returns the list of
        reduction results (NCDevArray; 0-d for full reductions), written into
        `red_out` (arrays of the right shape and dtype) when it is given."""
        reductions = list(reductions)
        t, _keep, ops, n = self._abi()
        stream = current_stream()
        if not reductions:
            if out is None:
                raise ValueError("nothing to evaluate")
            if out.size:
                _lib.call("nca_expr_eval", ctypes.byref(t), ops, n, ctypes.byref(out.view_struct()), stream)
            return []
        shape = out.shape if out is not None else self.shape
        results, rarr = _reductions(shape, self.expr_dtype, reductions, red_out)
        rs = list(rarr)
        if out is not None and out.size == 0:
            out = None
        _lib.call("nca_expr_reduce", ctypes.byref(t), ops, n,
                  ctypes.byref(out.view_struct()) if out is not None else None, rarr, len(rs), stream)
        return results

    # ---- host <-> device copies of views (nca_copy_host) ----
    def _host_view(self, host) -> _lib.View:
        """A View of a host numpy array or CPU torch tensor with this array's
        shape and itemsize (pinned torch memory makes the copy asynchronous)."""
        if isinstance(host, np.ndarray):
            ptr, itemsize, strides = host.ctypes.data, host.itemsize, tuple(host.strides)
        else:
            if host.is_cuda:
                raise TypeError("host buffer expected")
            itemsize = host.element_size()
            ptr, strides = host.data_ptr(), tuple(st * itemsize for st in host.stride())
        if tuple(host.shape) != tuple(self.shape) or itemsize != self.itemsize:
            raise ValueError(f"host buffer {tuple(host.shape)} x {itemsize} B does not match {self.shape} x "
                             f"{self.itemsize} B")
        return _lib.make_view(ptr, self.dtype, self.shape, strides)

    def copy_from(self, host, stream=None) -> "NCDevArray":
        """self[...] = host (same shape and itemsize) on `stream` (default: the
        current stream); both views contiguous along their innermost axis."""
        hv = self._host_view(host)
        _lib.call("nca_copy_host", ctypes.byref(hv), ctypes.byref(self.view_struct()),
                  current_stream() if stream is None else stream)
        return self

    def copy_to(self, host, stream=None) -> None:
        """host[...] = self (same shape and itemsize) on `stream`; asynchronous
        with pinned host memory (synchronise before reading it)."""
        hv = self._host_view(host)
        _lib.call("nca_copy_host", ctypes.byref(self.view_struct()), ctypes.byref(hv),
                  current_stream() if stream is None else stream)

    def __array__(self, dtype=None, copy=None):
        return self.materialize().__array__(dtype)

    def to_host(self) -> np.ndarray:
        return self.materialize().to_host()

    def _reduce(self, op: RedOp, axes):
        (res,) = self.evaluate(reductions=[(op, axes)])
        if axes is None:
            return _scalar(res)
        return res

    def sum(self, axes=None):
        return self._reduce(RedOp.SUM, axes)

    def mean(self, axes=None):
        return self._reduce(RedOp.MEAN, axes)

    def max(self, axes=None):
        return self._reduce(RedOp.MAX, axes)

    def min(self, axes=None):
        return self._reduce(RedOp.MIN, axes)

    def argmax(self, axes=None):
        return self._reduce(RedOp.ARGMAX, axes)

    def argmin(self, axes=None):
        return self._reduce(RedOp.ARGMIN, axes)


def _reductions(shape, expr_dtype: DType, reductions, red_out):
    """The result arrays of (RedOp, axes) reductions of a value of `shape` and
    their C descriptors (one shared axes mask)."""
    results, rs = [], []
    for i, (op, axes) in enumerate(reductions):
        op = RedOp(op)
        mask, kept = _axes_mask(axes, len(shape))
        odt = _red_out_dtype(op, expr_dtype)
        if red_out is not None:
            res = red_out[i]
            if res.dtype != odt or res.shape != tuple(shape[d] for d in kept):
                raise ValueError(f"reduction output {i} must be {odt.name} {[shape[d] for d in kept]}")
        else:
            res = NCDevArray([shape[d] for d in kept], odt)
        results.append(res)
        r = _lib.Reduction()
        r.op = int(op)
        r.axes_mask = mask
        r.out = res.view_struct()
        rs.append(r)
    if len({r.axes_mask for r in rs}) > 1:
        raise ValueError("one evaluate() call reduces over one set of axes")
    return results, (_lib.Reduction * max(len(rs), 1))(*rs)


def evaluate_many(outputs, reductions: Iterable = (), red_out=None):
    """Several expressions over shared operands in one pass (nca_expr_multi).

    `outputs` is a list of (expression, out array) pairs, all of one shape; the
    reductions (as in DevExpr.evaluate) apply to the first expression. The
    results equal evaluating the first expression with its reductions and then
    each further expression into its array; when the views allow it (operands
    staged by TMA, 4-byte outputs, no output overlapping an operand or another
    output) every operand is read once for all of them. Returns the reduction
    results."""
    outputs = list(outputs)
    if not outputs:
        raise ValueError("nothing to evaluate")
    exprs = [_as_node(e) for e, _ in outputs]
    outs = [o for _, o in outputs]
    shape = outs[0].shape
    for e, o in zip(exprs, outs):
        if o.shape != shape or e.shape != shape:
            raise ValueError("every expression and output must have the first output's shape")
    # one operand list: equal views become one operand, the tapes' loads are renumbered
    arrays, index = [], {}
    tapes = []
    for e in exprs:
        remap = []
        for a in e.arrays:
            k = _view_key(a)
            if k not in index:
                index[k] = len(arrays)
                arrays.append(a)
            remap.append(index[k])
        if remap != list(range(len(remap))):
            r = DevExpr()
            r.arrays, r.scalars, r.work, r.expr_dtype = [arrays[j] for j in remap], e.scalars, e.work, e.expr_dtype
            r.instrs = [((ins >> 24) << 24) | remap[ins & 0xFFFFFF]
                        if (ins >> 24) in (OpCode.LOAD_NCARR, OpCode.LOAD_SOARR) else ins for ins in e.instrs]
            e = r
        tapes.append(e._tape())
    reductions = list(reductions)
    results, rarr = _reductions(shape, exprs[0].expr_dtype, reductions, red_out)
    tarr = (_lib.Tape * len(tapes))(*[t for t, _ in tapes])
    ops = (_lib.View * max(len(arrays), 1))(*[a.view_struct() for a in arrays])
    oarr = (_lib.View * len(outs))(*[o.view_struct() for o in outs])
    if all(o.size for o in outs):
        _lib.call("nca_expr_multi", tarr, len(tapes), ops, len(arrays), oarr, rarr, len(reductions), current_stream())
    return results


def _view_key(a: NCDevArray):
    if a._ptr is not None:
        return (a.ptr, int(a.dtype), a.shape, a.strides, "ptr", a._ptr["poff"], a._ptr["step"])
    return (a.ptr, int(a.dtype), a.shape, a.strides)


def _axes_mask(axes, ndim: int):
    if axes is None:
        return (1 << ndim) - 1 if ndim < 32 else 0xFFFFFFFF, []
    if isinstance(axes, int):
        axes = [axes]
    mask = 0
    for a in axes:
        a = int(a)
        if a < 0:
            a += ndim
        if not 0 <= a < ndim:
            raise ValueError("axis out of range")
        mask |= 1 << a
    kept = [d for d in range(ndim) if not (mask >> d) & 1]
    return mask, kept


def _red_out_dtype(op: RedOp, dt: DType) -> DType:
    if op == RedOp.SUM:
        return sum_type(dt)
    if op == RedOp.MEAN:
        return DType.float64
    if op in (RedOp.MAX, RedOp.MIN):
        return arith(dt)
    return DType.int64


def _scalar(a: NCDevArray):
    v = a.to_host().reshape(-1)[0]
    if a.dtype == DType.bool:
        return bool(v)
    if a.dtype in FLOATS:
        return float(v)
    return int(v)


# ---- operators on arrays and expressions ------------------------------------------
def _def_ops(cls):
    binops = {
        "add": OpCode.ADD, "sub": OpCode.SUB, "mul": OpCode.MUL, "truediv": OpCode.DIV,
        "mod": OpCode.MOD, "and": OpCode.BAND, "or": OpCode.BOR, "xor": OpCode.XOR,
    }
    for name, op in binops.items():
        def f(self, other, _op=op):
            return _as_node(self)._binary(_op, other)

        def rf(self, other, _op=op):
            return _as_node(self)._binary(_op, other, reverse=True)
        setattr(cls, f"__{name}__", f)
        setattr(cls, f"__r{name}__", rf)
    cmps = {"eq": OpCode.EQ, "ne": OpCode.NE, "lt": OpCode.LT, "le": OpCode.LE, "gt": OpCode.GT, "ge": OpCode.GE}
    for name, op in cmps.items():
        def c(self, other, _op=op):
            return _as_node(self)._binary(_op, other)
        setattr(cls, f"__{name}__", c)
    cls.__neg__ = lambda self: _as_node(self)._unary(OpCode.NEG)
    cls.__abs__ = lambda self: _as_node(self)._unary(OpCode.ABS)
    cls.__invert__ = lambda self: _as_node(self)._unary(OpCode.BNOT)
    cls.__hash__ = object.__hash__


_def_ops(NCDevArray)
_def_ops(DevExpr)


def _inplace(name, op):
    def f(self, other):
        with lazy_mode():
            e = _as_node(self)._binary(op, other)
        e.evaluate(out=self)
        return self
    setattr(NCDevArray, f"__i{name}__", f)


for _n, _o in (("add", OpCode.ADD), ("sub", OpCode.SUB), ("mul", OpCode.MUL), ("truediv", OpCode.DIV),
               ("mod", OpCode.MOD)):
    _inplace(_n, _o)


def sqrt(x):
    return _as_node(x)._unary(OpCode.SQRT)


def absolute(x):
    return _as_node(x)._unary(OpCode.ABS)


def inc(x):
    """x + 1 in x's dtype (ncarray's INC opcode)."""
    return _as_node(x)._unary(OpCode.INC)


def dec(x):
    """x - 1 in x's dtype (ncarray's DEC opcode)."""
    return _as_node(x)._unary(OpCode.DEC)


def logical_and(a, b):
    return _as_node(a)._binary(OpCode.LAND, b)


def logical_or(a, b):
    return _as_node(a)._binary(OpCode.LOR, b)


def logical_not(a):
    return _as_node(a)._unary(OpCode.LNOT)


def iota(like, dtype: DType = DType.int64):
    e = DevExpr.iota(like, dtype)
    return e._finish()
