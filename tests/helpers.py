"""Shared helpers of the parity tests: seeded inputs in every dtype and
bit-level comparison against the oracle."""
from __future__ import annotations

import numpy as np

from ncarray_gb300.dtype import DType, ITEMSIZE, compute_dtype

SEED = 20261203


def rand(rng: np.random.Generator, shape, dt: DType) -> np.ndarray:
    """Seeded host data of ncarray dtype `dt` (bfloat16 as uint16 bit patterns)."""
    dt = DType(dt)
    if dt == DType.bool:
        return rng.integers(0, 2, shape).astype(np.bool_)
    if dt in (DType.int8, DType.char):
        return rng.integers(-128, 128, shape).astype(np.int8)
    if dt == DType.uint8:
        return rng.integers(0, 256, shape).astype(np.uint8)
    if dt == DType.int16:
        return rng.integers(-30000, 30000, shape).astype(np.int16)
    if dt == DType.uint16:
        return rng.integers(0, 65536, shape).astype(np.uint16)
    if dt == DType.int32:
        return rng.integers(-1000, 1001, shape).astype(np.int32)
    if dt == DType.uint32:
        return rng.integers(0, 2**32, shape, dtype=np.uint64).astype(np.uint32)
    if dt == DType.int64:
        return rng.integers(-2**40, 2**40, shape).astype(np.int64)
    if dt == DType.uint64:
        return rng.integers(0, 2**62, shape, dtype=np.uint64)
    if dt == DType.float32:
        return rng.normal(size=shape).astype(np.float32)
    if dt == DType.float64:
        return rng.uniform(-1, 1, shape)
    if dt == DType.float16:
        return rng.normal(size=shape).astype(np.float16)
    if dt == DType.bfloat16:
        f = rng.normal(size=shape).astype(np.float32)
        return (f.view(np.uint32) >> 16).astype(np.uint16)
    raise ValueError(dt)


def bits(a: np.ndarray) -> np.ndarray:
    """Integer view of the bytes (exact comparison, NaN payloads included)."""
    a = np.ascontiguousarray(a)
    return a.view({1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[a.itemsize])


def assert_bits_equal(got: np.ndarray, want: np.ndarray, what: str = "") -> None:
    assert got.shape == want.shape, f"{what}: shape {got.shape} != {want.shape}"
    assert got.dtype.itemsize == want.dtype.itemsize
    g, w = bits(got), bits(want)
    bad = np.flatnonzero(g.reshape(-1) != w.reshape(-1))
    assert bad.size == 0, (f"{what}: {bad.size} of {g.size} elements differ, first at {bad[:5]}: "
                           f"got {got.reshape(-1)[bad[:5]]} want {want.reshape(-1)[bad[:5]]}")


def oracle_eval(orc, expr, host_ops):
    """Evaluates a DevExpr's tape on the host operands with the oracle."""
    assert len(host_ops) == len(expr.arrays), "one host operand per tape operand"
    return orc.expr_eval(expr.instrs, expr.scalars, int(compute_dtype(expr.expr_dtype, expr.work)),
                         [(h, int(a.dtype)) for h, a in zip(host_ops, expr.arrays)], expr.shape,
                         int(expr.expr_dtype))
