"""Python access to the oracle (TEST INFRASTRUCTURE ONLY).

``liboracle.so``  -- the C restatement of the reference algorithms (oracle.c).
``libncref.so``   -- ncarray's own host code compiled from its sources
                     (oracle/_ref, built only where the reference is present).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the oracle (never as the thing measured or shipped).
"""
from __future__ import annotations

import ctypes
import subprocess
from ctypes import POINTER, c_double, c_float, c_int, c_int32, c_int64, c_uint32, c_uint64, c_void_p
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libncref.so"

ITEMSIZE = {0: 1, 1: 1, 2: 1, 3: 2, 4: 4, 5: 8, 6: 1, 7: 2, 8: 4, 9: 8, 10: 4, 11: 8, 22: 2, 23: 2}


class OrcView(ctypes.Structure):
    _fields_ = [
        ("data", c_void_p), ("dtype", c_int32), ("ndim", c_int32), ("shape", c_int64 * 10),
        ("strides", c_int64 * 10), ("offsets", c_int64 * 10), ("pointer_axis", c_int32), ("flags", c_int32),
    ]


class OrcItem(ctypes.Structure):
    _fields_ = [("data", c_void_p), ("length", c_int64), ("dtype", c_int32), ("reserved", c_int32)]


class OrcResult(ctypes.Structure):
    _fields_ = [("sum", c_double), ("mean", c_double), ("max", c_double), ("sum_sq_m", c_double)]


def build(with_ref: Optional[bool] = None) -> None:
    """Builds liboracle.so, and libncref.so when the reference sources exist
    (their location is the Makefile's REF, or NCA_REFERENCE_DIR)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "oracle"], check=True)
    if with_ref is None:
        with_ref = subprocess.run(["make", "-s", "-C", str(HERE), "have-ref"],
                                  capture_output=True).returncode == 0
    if with_ref:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref"], check=True)


_orc = None
_ref = None


def lib() -> ctypes.CDLL:
    global _orc
    if _orc is None:
        if not LIB.exists():
            build(with_ref=False)
        L = ctypes.CDLL(str(LIB))
        L.orc_expr_eval.argtypes = [POINTER(c_uint32), c_int, POINTER(c_int), POINTER(c_uint64), c_int, c_int,
                                    POINTER(OrcView), c_int, POINTER(OrcView)]
        L.orc_reduce.argtypes = [POINTER(OrcView), c_int, c_uint32, POINTER(OrcView)]
        L.orc_stencil3d_f64.argtypes = [POINTER(c_double), c_int64, c_int64, c_int64, POINTER(c_double), c_double, c_int]
        L.orc_hist2d.argtypes = [c_void_p, c_void_p, c_void_p, c_int64, c_int, c_int, c_double, c_double, c_double,
                                 c_double, c_void_p, c_void_p]
        L.orc_batch_reduce.argtypes = [POINTER(OrcItem), c_int, POINTER(OrcResult), c_int]
        L.orc_scatter_add.argtypes = [POINTER(OrcView), POINTER(OrcView), POINTER(OrcView)]
        _orc = L
    return _orc


def ref() -> Optional[ctypes.CDLL]:
    """The reference's own host code, or None where it was not built."""
    global _ref
    if _ref is None and REF_LIB.exists():
        L = ctypes.CDLL(str(REF_LIB))
        L.ref_last_error.restype = ctypes.c_char_p
        _ref = L
    return _ref


def view_of(a: np.ndarray, dtype: int) -> OrcView:
    v = OrcView()
    v.data = a.ctypes.data if a.size else None
    v.dtype = dtype
    v.ndim = a.ndim
    for d in range(a.ndim):
        v.shape[d] = a.shape[d]
        v.strides[d] = a.strides[d]
        v.offsets[d] = 0
    v.pointer_axis = -1
    v.flags = 0
    return v


def np_dtype(dt: int):
    return {0: np.bool_, 1: np.int8, 2: np.uint8, 3: np.uint16, 4: np.uint32, 5: np.uint64, 6: np.int8,
            7: np.int16, 8: np.int32, 9: np.int64, 10: np.float32, 11: np.float64, 22: np.uint16,
            23: np.float16}[dt]


def expr_eval(instrs: Sequence[int], scalars: Sequence[tuple], compute_dtype: int,
              operands: Sequence[tuple], out_shape: Sequence[int], out_dtype: int) -> np.ndarray:
    """operands: (numpy array, ncarray dtype) pairs; scalars: (dtype, slot) pairs."""
    out = np.zeros(tuple(out_shape), dtype=np_dtype(out_dtype))
    ins = (c_uint32 * max(len(instrs), 1))(*instrs)
    sd = (c_int * max(len(scalars), 1))(*[d for d, _ in scalars])
    ss = (c_uint64 * max(len(scalars), 1))(*[s for _, s in scalars])
    views = (OrcView * max(len(operands), 1))(*[view_of(a, d) for a, d in operands])
    ov = view_of(out, out_dtype)
    rc = lib().orc_expr_eval(ins, len(instrs), sd, ss, len(scalars), compute_dtype, views, len(operands),
                             ctypes.byref(ov))
    if rc:
        raise RuntimeError(f"oracle expr_eval failed ({rc})")
    return out


SUM_DT = {0: 5, 2: 5, 3: 5, 6: 9, 7: 9, 22: 10, 23: 10}


def red_out_dtype(op: int, dt: int) -> int:
    if op == 0:
        return SUM_DT.get(dt, dt)
    if op == 1:
        return 11
    if op in (2, 3):
        return 10 if dt in (22, 23) else dt
    return 9


def reduce(a: np.ndarray, dtype: int, op: int, axes=None) -> np.ndarray:
    """Reduction of `a` (ncarray dtype `dtype`) over `axes` (None = all)."""
    n = a.ndim
    if axes is None:
        mask = (1 << n) - 1
    else:
        axes = [axes] if isinstance(axes, int) else list(axes)
        mask = 0
        for x in axes:
            mask |= 1 << (x % n if n else 0)
    kept = [a.shape[d] for d in range(n) if not (mask >> d) & 1]
    odt = red_out_dtype(op, dtype)
    out = np.zeros(tuple(kept), dtype=np_dtype(odt))
    rc = lib().orc_reduce(ctypes.byref(view_of(a, dtype)), op, mask, ctypes.byref(view_of(out, odt)))
    if rc:
        raise RuntimeError("oracle reduce failed")
    return out


def stencil3d_f64(u: np.ndarray, weights27: Sequence[float], dt: float, iters: int) -> np.ndarray:
    out = np.ascontiguousarray(u, dtype=np.float64).copy()
    w = (c_double * 27)(*weights27)
    nz, ny, nx = out.shape
    rc = lib().orc_stencil3d_f64(out.ctypes.data_as(POINTER(c_double)), nz, ny, nx, w, dt, iters)
    if rc:
        raise RuntimeError("oracle stencil failed")
    return out


def hist2d(x, y, w, nbx, nby, x_lo, x_hi, y_lo, y_hi):
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    counts = np.zeros(nbx * nby, dtype=np.uint64)
    wsum = np.zeros(nbx * nby, dtype=np.float64) if w is not None else None
    wp = np.ascontiguousarray(w, dtype=np.float32) if w is not None else None
    lib().orc_hist2d(x.ctypes.data, y.ctypes.data, wp.ctypes.data if wp is not None else None, x.size, nbx, nby,
                     x_lo, x_hi, y_lo, y_hi, counts.ctypes.data, wsum.ctypes.data if wsum is not None else None)
    return counts, wsum


def batch_reduce(arrays: Sequence[np.ndarray], dtypes: Sequence[int], nthreads: int = 1) -> np.ndarray:
    """Per array (sum, mean, max, sum(x*x-x)) in float64; arrays are 1-D numpy
    buffers (bfloat16 as uint16 bit patterns)."""
    items = (OrcItem * len(arrays))()
    for i, (a, d) in enumerate(zip(arrays, dtypes)):
        items[i].data = a.ctypes.data
        items[i].length = a.size
        items[i].dtype = d
    res = (OrcResult * len(arrays))()
    lib().orc_batch_reduce(items, len(arrays), res, nthreads)
    return np.array([[r.sum, r.mean, r.max, r.sum_sq_m] for r in res], dtype=np.float64)


def scatter_add(dest: np.ndarray, dest_dtype: int, idx: np.ndarray, idx_dtype: int, src: np.ndarray,
                src_dtype: int) -> np.ndarray:
    """dest (1-D, updated in place and returned) += src scattered by idx, in
    the reference's order and arithmetic (host::scatter_add_recursive)."""
    rc = lib().orc_scatter_add(ctypes.byref(view_of(dest, dest_dtype)), ctypes.byref(view_of(idx, idx_dtype)),
                               ctypes.byref(view_of(src, src_dtype)))
    if rc:
        raise RuntimeError(f"oracle scatter_add failed ({rc})")
    return dest


# ---- the reference's own implementation (oracle/_ref) -------------------------------
def ref_expr_eval(instrs, scalars, work_dtype: int, expr_dtype: int, operands, out_shape):
    L = ref()
    if L is None:
        return None
    n = len(operands)
    data = (c_void_p * max(n, 1))(*[a.ctypes.data for a, _ in operands])
    dts = (c_int * max(n, 1))(*[d for _, d in operands])
    nds = (c_int * max(n, 1))(*[a.ndim for a, _ in operands])
    shapes = (c_int64 * (10 * max(n, 1)))()
    strides = (c_int64 * (10 * max(n, 1)))()
    for k, (a, _) in enumerate(operands):
        for d in range(a.ndim):
            shapes[10 * k + d] = a.shape[d]
            strides[10 * k + d] = a.strides[d]
    out = np.zeros(tuple(out_shape), dtype=np_dtype(expr_dtype))
    ins = (c_uint32 * len(instrs))(*instrs)
    sd = (c_int * max(len(scalars), 1))(*[d for d, _ in scalars])
    ss = (c_uint64 * max(len(scalars), 1))(*[s for _, s in scalars])
    osh = (c_int64 * len(out_shape))(*out_shape)
    rc = L.ref_expr_eval(ins, len(instrs), n, data, dts, nds, shapes, strides, len(scalars), sd, ss, work_dtype,
                         expr_dtype, c_void_p(out.ctypes.data), len(out_shape), osh)
    if rc:
        raise RuntimeError(L.ref_last_error().decode())
    return out


def ref_reduce_full(a: np.ndarray, dtype: int, op: int):
    L = ref()
    if L is None:
        return None
    sh = (c_int64 * max(a.ndim, 1))(*a.shape)
    st = (c_int64 * max(a.ndim, 1))(*a.strides)
    buf = (ctypes.c_uint8 * 8)()
    odt = c_int(0)
    rc = L.ref_reduce_full(c_void_p(a.ctypes.data), dtype, a.ndim, sh, st, op, buf, ctypes.byref(odt))
    if rc:
        raise RuntimeError(L.ref_last_error().decode())
    return np.frombuffer(bytes(buf)[: ITEMSIZE[odt.value]], dtype=np_dtype(odt.value))[0], odt.value


def ref_reduce_axes(a: np.ndarray, dtype: int, op: int, axes):
    L = ref()
    if L is None:
        return None
    axes = [axes] if isinstance(axes, int) else list(axes)
    mask = 0
    for x in axes:
        mask |= 1 << x
    sh = (c_int64 * a.ndim)(*a.shape)
    st = (c_int64 * a.ndim)(*a.strides)
    cap = a.size * 8 + 64
    buf = (ctypes.c_uint8 * cap)()
    odt, on = c_int(0), c_int64(0)
    rc = L.ref_reduce_axes(c_void_p(a.ctypes.data), dtype, a.ndim, sh, st, c_uint32(mask), op, buf, c_int64(cap),
                           ctypes.byref(odt), ctypes.byref(on))
    if rc:
        raise RuntimeError(L.ref_last_error().decode())
    kept = [a.shape[d] for d in range(a.ndim) if not (mask >> d) & 1]
    nbytes = on.value * ITEMSIZE[odt.value]
    return np.frombuffer(bytes(buf)[:nbytes], dtype=np_dtype(odt.value)).reshape(kept), odt.value


def ref_scatter_add(dest: np.ndarray, dest_dtype: int, idx: np.ndarray, idx_dtype: int, src: np.ndarray,
                    src_dtype: int):
    """dest += src scattered by idx through the reference's own
    host::scatter_add_recursive; None where oracle/_ref was not built."""
    L = ref()
    if L is None:
        return None
    n = src.ndim
    sh = (c_int64 * max(n, 1))(*src.shape)
    ist = (c_int64 * max(n, 1))(*idx.strides)
    sst = (c_int64 * max(n, 1))(*src.strides)
    rc = L.ref_scatter_add(c_void_p(dest.ctypes.data), dest_dtype, c_int64(dest.shape[0]), c_int64(dest.strides[0]),
                           c_void_p(idx.ctypes.data), idx_dtype, c_void_p(src.ctypes.data), src_dtype, n, sh, ist,
                           sst)
    if rc:
        raise RuntimeError(L.ref_last_error().decode())
    return dest
