"""ctypes binding of libncgb300 (include/ncgb300.h).

The library is built in-tree by ``ncarray_gb300.build``. Importing the device
API without it raises: there is no CPU fallback on the device path.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_float, c_int32, c_int64, c_uint32, c_uint64, c_void_p
from pathlib import Path

MAX_NDIM = 10
LIB_PATH = Path(__file__).resolve().parent / "_build" / "libncgb300.so"

# status codes
OK, ERR_INVALID, ERR_DTYPE, ERR_SHAPE, ERR_COMPILE, ERR_CUDA, ERR_OOM, ERR_TIMEOUT, ERR_UNSUPPORTED, ERR_LIMIT = range(10)
STATUS_NAMES = {
    0: "OK", 1: "INVALID", 2: "DTYPE", 3: "SHAPE", 4: "COMPILE", 5: "CUDA", 6: "OOM",
    7: "TIMEOUT", 8: "UNSUPPORTED", 9: "LIMIT",
}


class NcaError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{STATUS_NAMES.get(status, status)}] {message}")
        self.status = status


class View(ctypes.Structure):
    _fields_ = [
        ("data", c_void_p),
        ("dtype", c_int32),
        ("ndim", c_int32),
        ("shape", c_int64 * MAX_NDIM),
        ("strides", c_int64 * MAX_NDIM),
        ("offsets", c_int64 * MAX_NDIM),
        ("pointer_axis", c_int32),
        ("flags", c_int32),
    ]


class Tape(ctypes.Structure):
    _fields_ = [
        ("instrs", POINTER(c_uint32)),
        ("n_instrs", c_int32),
        ("n_scalars", c_int32),
        ("scalar_dtypes", POINTER(c_int32)),
        ("scalar_slots", POINTER(c_uint64)),
        ("compute_dtype", c_int32),
        ("result_dtype", c_int32),
    ]


class Reduction(ctypes.Structure):
    _fields_ = [("op", c_int32), ("axes_mask", c_uint32), ("out", View)]


class BatchItem(ctypes.Structure):
    _fields_ = [("data", c_void_p), ("length", c_int64), ("dtype", c_int32), ("reserved", c_int32)]


BATCH_MAX_OUTS = 4


class BatchExprItem(ctypes.Structure):
    _fields_ = [("data", c_void_p), ("length", c_int64), ("dtype", c_int32), ("n_outs", c_int32),
                ("tape", c_int32 * BATCH_MAX_OUTS), ("op", c_int32 * BATCH_MAX_OUTS)]


class BatchValue(ctypes.Structure):
    _fields_ = [("value", c_double), ("index", c_int64)]


class BatchResult(ctypes.Structure):
    _fields_ = [("sum", c_double), ("mean", c_double), ("max", c_double), ("sum_sq_m", c_double)]


EXPORTS = {
    "nca_last_error": (c_char_p, []),
    "nca_version": (c_int32, []),
    "nca_launch_count": (c_int64, []),
    "nca_device_status": (c_int32, [POINTER(c_int32), c_void_p]),
    "nca_wait_probe": (c_int32, [c_double, c_void_p]),
    "nca_tune_set_mode": (c_int32, [c_int32]),
    "nca_tune_get": (c_int32, [c_char_p, POINTER(c_int32), c_int32, POINTER(c_int32)]),
    "nca_tune_clear": (c_int32, []),
    "nca_jit_stats": (c_int32, [POINTER(c_int64), POINTER(c_int64), POINTER(c_int64)]),
    "nca_jit_set_cache_dir": (c_int32, [c_char_p]),
    "nca_jit_selftest": (c_int32, [c_char_p, POINTER(c_int32)]),
    "nca_expr_eval": (c_int32, [POINTER(Tape), POINTER(View), c_int32, POINTER(View), c_void_p]),
    "nca_expr_reduce": (c_int32, [POINTER(Tape), POINTER(View), c_int32, POINTER(View), POINTER(Reduction), c_int32, c_void_p]),
    "nca_expr_multi": (c_int32, [POINTER(Tape), c_int32, POINTER(View), c_int32, POINTER(View), POINTER(Reduction),
                                 c_int32, c_void_p]),
    "nca_reduce": (c_int32, [POINTER(View), c_int32, c_uint32, POINTER(View), c_void_p]),
    "nca_reduce_noalloc": (c_int32, [POINTER(View), c_int32, POINTER(View), c_void_p]),
    "nca_copy": (c_int32, [POINTER(View), POINTER(View), c_void_p]),
    "nca_copy_host": (c_int32, [POINTER(View), POINTER(View), c_void_p]),
    "nca_fill": (c_int32, [POINTER(View), c_int32, c_void_p, c_void_p]),
    "nca_stencil3d": (c_int32, [POINTER(View), POINTER(View), POINTER(c_double), c_double, c_void_p]),
    "nca_stencil3d_iterate": (c_int32, [POINTER(View), POINTER(View), POINTER(c_double), c_double, c_int32, c_void_p]),
    "nca_hist2d": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_int32, c_int32, c_double, c_double,
                             c_double, c_double, c_void_p, c_void_p, c_void_p]),
    "nca_stencil": (c_int32, [POINTER(View), POINTER(View), POINTER(c_int64), c_int32, POINTER(Tape), c_void_p]),
    "nca_scatter_add": (c_int32, [POINTER(View), POINTER(View), POINTER(View), c_void_p]),
    "nca_batch_create": (c_int32, [POINTER(BatchItem), c_int32, POINTER(c_void_p), c_void_p]),
    "nca_batch_reduce": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "nca_batch_reduce_graph": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "nca_batch_reduce_plain": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "nca_batch_autotune": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "nca_batch_schedule": (c_int32, [c_void_p, POINTER(c_int64), POINTER(c_int32), POINTER(c_int32), POINTER(c_int32)]),
    "nca_batch_status": (c_int32, [c_void_p, POINTER(c_int32), c_void_p]),
    "nca_batch_destroy": (None, [c_void_p]),
    "nca_batch_expr_create": (c_int32, [POINTER(BatchExprItem), c_int32, POINTER(Tape), c_int32, POINTER(c_void_p), c_void_p]),
    "nca_batch_expr_run": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "nca_batch_expr_run_graph": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "nca_batch_expr_run_plain": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "nca_batch_expr_info": (c_int32, [c_void_p, POINTER(c_int64), POINTER(c_int32), POINTER(c_int32)]),
    "nca_batch_expr_destroy": (None, [c_void_p]),
}

_lib = None


def lib() -> ctypes.CDLL:
    """Loads the library (once). Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m ncarray_gb300.build` "
                "(there is no CPU fallback on the device path)")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in EXPORTS.items():
            if hasattr(L, name):
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != OK:
        msg = lib().nca_last_error()
        raise NcaError(status, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))


VIEW_SUBOFFSETS = 1   # nca_view.flags: PEP 3118 suboffset semantics on the pointer axis


def make_view(ptr: int, dtype: int, shape, byte_strides, byte_offset: int = 0) -> View:
    v = View()
    v.data = ptr + byte_offset if ptr else None
    v.dtype = int(dtype)
    v.ndim = len(shape)
    if v.ndim > MAX_NDIM:
        raise ValueError(f"at most {MAX_NDIM} dims")
    for d, (n, s) in enumerate(zip(shape, byte_strides)):
        v.shape[d] = int(n)
        v.strides[d] = int(s)
        v.offsets[d] = 0
    v.pointer_axis = -1
    v.flags = 0
    return v
