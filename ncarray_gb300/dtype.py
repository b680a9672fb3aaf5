"""ncarray dtypes and the expression type rules.

Numbering follows ncarray::DType (src/lib/ncarray/dtype.hh:56-80); bfloat16
and float16 are appended storage types that compute as float32.
Type rules restated from:
  - promote_expr_types: larger enum wins (expression/interface.hh:91-100)
  - determine_dtype_for_op (op_code.hh:101-161) with op_traits sum_type /
    diff_type / truediv_type (op_traits.hh:72-76,380-410)
"""
from __future__ import annotations

import enum

import numpy as np


class DType(enum.IntEnum):
    bool = 0
    char = 1
    uint8 = 2
    uint16 = 3
    uint32 = 4
    uint64 = 5
    int8 = 6
    int16 = 7
    int32 = 8
    int64 = 9
    float32 = 10
    float64 = 11
    bfloat16 = 22
    float16 = 23


class OpCode(enum.IntEnum):
    NOOP = 0
    IDX = 1
    LOAD_NCARR = 2
    LOAD_SOARR = 3
    LOAD_CONST = 4
    NEG = 5
    INC = 6
    DEC = 7
    LNOT = 12
    BNOT = 13
    ADD = 14
    SUB = 15
    MUL = 16
    DIV = 17
    MOD = 18
    EQ = 20
    NE = 21
    LT = 22
    LE = 23
    GT = 24
    GE = 25
    LAND = 26
    LOR = 27
    BAND = 28
    BOR = 29
    XOR = 30
    ABS = 34
    SQRT = 35


class RedOp(enum.IntEnum):
    SUM = 0
    MEAN = 1
    MAX = 2
    MIN = 3
    ARGMAX = 4
    ARGMIN = 5


ITEMSIZE = {
    DType.bool: 1, DType.char: 1, DType.uint8: 1, DType.uint16: 2, DType.uint32: 4,
    DType.uint64: 8, DType.int8: 1, DType.int16: 2, DType.int32: 4, DType.int64: 8,
    DType.float32: 4, DType.float64: 8, DType.bfloat16: 2, DType.float16: 2,
}

FLOATS = {DType.float32, DType.float64, DType.bfloat16, DType.float16}
SIGNED = {DType.char, DType.int8, DType.int16, DType.int32, DType.int64} | FLOATS

_NP = {
    DType.bool: np.bool_, DType.char: np.int8, DType.uint8: np.uint8, DType.uint16: np.uint16,
    DType.uint32: np.uint32, DType.uint64: np.uint64, DType.int8: np.int8, DType.int16: np.int16,
    DType.int32: np.int32, DType.int64: np.int64, DType.float32: np.float32,
    DType.float64: np.float64, DType.float16: np.float16,
}


def to_numpy(dt: DType):
    """numpy dtype holding the bytes of `dt` (bfloat16 -> uint16 bit patterns)."""
    dt = DType(dt)
    if dt == DType.bfloat16:
        return np.dtype(np.uint16)
    return np.dtype(_NP[dt])


def from_numpy(npdt) -> DType:
    npdt = np.dtype(npdt)
    for k, v in _NP.items():
        if k == DType.char:
            continue
        if np.dtype(v) == npdt:
            return k
    raise TypeError(f"numpy dtype {npdt} has no ncarray counterpart")


def arith(dt: DType) -> DType:
    """float32 stands in for the 16-bit float storage types in arithmetic."""
    return DType.float32 if dt in (DType.bfloat16, DType.float16) else DType(dt)


def promote(a: DType, b: DType) -> DType:
    """promote_expr_types: the numerically larger DType."""
    a, b = arith(a), arith(b)
    return a if int(a) >= int(b) else b


def sum_type(dt: DType) -> DType:
    dt = DType(dt)
    if dt in (DType.bool, DType.uint8, DType.uint16):
        return DType.uint64
    if dt in (DType.int8, DType.int16):
        return DType.int64
    return arith(dt)


def diff_type(dt: DType) -> DType:
    dt = DType(dt)
    if dt in (DType.bool, DType.uint8, DType.uint16, DType.int8, DType.int16):
        return DType.int64
    return arith(dt)


def result_dtype(op: OpCode, work: DType) -> DType:
    """determine_dtype_for_op(op, work)."""
    work = arith(work)
    if op in (OpCode.LNOT, OpCode.EQ, OpCode.NE, OpCode.LT, OpCode.LE, OpCode.GT, OpCode.GE,
              OpCode.LAND, OpCode.LOR):
        return DType.bool
    if op == OpCode.ADD:
        return sum_type(work)
    if op == OpCode.SUB:
        return diff_type(work)
    if op == OpCode.DIV:
        return DType.float64
    if op == OpCode.SQRT and work not in FLOATS:
        return DType.float64
    return work


def compute_dtype(expr_dt: DType, work: DType) -> DType:
    """The VM's WorkT: the result dtype, or the work dtype for bool results."""
    return arith(work) if expr_dt == DType.bool else arith(expr_dt)


def scalar_dtype(value) -> DType:
    """DType a Python scalar takes in ncarray's bindings (the first alternative of
    the Scalar variant that accepts it without conversion: dtype.hh:213-225)."""
    if isinstance(value, (bool, np.bool_)):
        return DType.bool
    if isinstance(value, np.generic):
        return from_numpy(value.dtype)
    if isinstance(value, int):
        for dt, lo, hi in ((DType.uint8, 0, 2**8 - 1), (DType.uint16, 0, 2**16 - 1),
                           (DType.uint32, 0, 2**32 - 1), (DType.uint64, 0, 2**64 - 1),
                           (DType.int8, -2**7, 2**7 - 1), (DType.int16, -2**15, 2**15 - 1),
                           (DType.int32, -2**31, 2**31 - 1), (DType.int64, -2**63, 2**63 - 1)):
            if lo <= value <= hi:
                return dt
        raise OverflowError("integer scalar out of 64-bit range")
    if isinstance(value, float):
        return DType.float32
    raise TypeError(f"unsupported scalar {value!r}")


def scalar_slot(value, dt: DType) -> int:
    """8-byte slot carrying `value` as dtype `dt`."""
    dt = DType(dt)
    if dt == DType.bfloat16:
        b = np.array([value], dtype=np.float32).view(np.uint32)[0] >> 16
        return int(b)
    arr = np.zeros(1, dtype=np.uint64)
    raw = np.array([value]).astype(to_numpy(dt)).tobytes()
    arr.view(np.uint8)[: len(raw)] = np.frombuffer(raw, dtype=np.uint8)
    return int(arr[0])
