"""ncarray_gb300: the data-parallel device path of ncarray, rebuilt for GB300 (sm_103a).

Public surface (mirrors ncarray's ``_pyncdevarray`` for device arrays):
  NCDevArray, DevExpr, DType, OpCode, RedOp, set_eager, lazy_mode, sqrt,
  absolute, iota, inc, dec, logical_and/or/not, evaluate_many (several
  expressions over shared operands in one pass), and the stencil, histogram
  and batched reduction entry points.
"""
from .dtype import DType, OpCode, RedOp
from .array import (NCDevArray, DevExpr, set_eager, lazy_mode, sqrt, absolute, iota, inc, dec, logical_and,
                    logical_or, logical_not, current_stream, evaluate_many)
from ._lib import NcaError

__all__ = [
    "DType", "OpCode", "RedOp", "NCDevArray", "DevExpr", "set_eager", "lazy_mode", "sqrt",
    "absolute", "iota", "inc", "dec", "logical_and", "logical_or", "logical_not", "current_stream", "evaluate_many", "NcaError",
]
